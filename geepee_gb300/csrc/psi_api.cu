// C ABI of the psi-statistics kernels (see psi_impl.cuh for the algorithm).
#include "psi_impl.cuh"

int psi_fwd_df64(const psi_impl::PsiArgs<double>& a, cudaStream_t st);
int psi_bwd_df64(const psi_impl::PsiArgs<double>& a, cudaStream_t st);
int psi_fwd_f32(const psi_impl::PsiArgs<float>& a, cudaStream_t st);
int psi_bwd_f32(const psi_impl::PsiArgs<float>& a, cudaStream_t st);
using psi_impl::QMAX;
using psi_impl::DMAX;

template <typename S>
static psi_impl::PsiArgs<S> make_args(int N, int M, int Q, int Dout, const void* mu, const void* var, const void* Z,
                     const double* lls2, const double* lsf2, const void* A, const void* B) {
  psi_impl::PsiArgs<S> a{};
  a.N = N; a.M = M; a.Q = Q; a.Dout = Dout;
  a.mu = (const S*)mu; a.var = (const S*)var; a.Z = (const S*)Z;
  a.lls2 = lls2; a.lsf2 = lsf2;
  a.A = (const S*)A; a.B = (const S*)B;
  return a;
}


extern "C" int gpk_psi_fwd(int prec, int N, int M, int Q, int Dout, const void* mu, const void* var,
                           const void* Z, const double* lls2, const double* lsf2, const void* A,
                           const void* B, void* psi1, void* psi2, double* psi2_sum, void* m_out,
                           void* v_out, void* stream) {
  GPK_NVTX("gpk_psi_fwd");
  GPK_REQUIRE(N >= 0 && M >= 1 && Q >= 1 && Q <= QMAX, "psi_fwd: bad sizes N=%d M=%d Q=%d", N, M, Q);
  GPK_REQUIRE(Dout >= 0 && Dout <= DMAX, "psi_fwd: Dout=%d outside [0,%d]", Dout, DMAX);
  GPK_REQUIRE(mu && var && Z && lls2 && lsf2, "psi_fwd: null input");
  GPK_REQUIRE(!(m_out || v_out) || (A && B && Dout >= 1), "psi_fwd: m/v need A, B and Dout >= 1");
  cudaStream_t st = gpk::as_stream(stream);
  if (prec == GPK_DF64) {
    auto a = make_args<double>(N, M, Q, Dout, mu, var, Z, lls2, lsf2, A, B);
    a.psi1 = (double*)psi1; a.psi2 = (double*)psi2; a.psi2_sum = psi2_sum;
    a.m_out = (double*)m_out; a.v_out = (double*)v_out;
    return psi_fwd_df64(a, st);
  } else if (prec == GPK_FP32) {
    auto a = make_args<float>(N, M, Q, Dout, mu, var, Z, lls2, lsf2, A, B);
    a.psi1 = (float*)psi1; a.psi2 = (float*)psi2; a.psi2_sum = psi2_sum;
    a.m_out = (float*)m_out; a.v_out = (float*)v_out;
    return psi_fwd_f32(a, st);
  }
  return gpk::fail(GPK_EINVAL, "psi_fwd: unknown precision %d", prec);
}

extern "C" int gpk_psi_rollout(int prec, int T, int M, int Q, const void* mu0, const void* var0, const void* Z,
                               const double* lls2, const double* lsf2, const void* A, const void* B, void* m_out,
                               void* v_out, void* stream) {
  GPK_NVTX("gpk_psi_rollout");
  GPK_REQUIRE(T >= 0 && M >= 1 && Q >= 1 && Q <= DMAX && Q <= QMAX, "psi_rollout: bad sizes T=%d M=%d Q=%d", T, M, Q);
  GPK_REQUIRE(mu0 && var0 && Z && lls2 && lsf2 && A && B && m_out && v_out, "psi_rollout: null pointer");
  cudaStream_t st = gpk::as_stream(stream);
  if (prec == GPK_DF64) {
    auto a = make_args<double>(T, M, Q, Q, mu0, var0, Z, lls2, lsf2, A, B);
    a.m_out = (double*)m_out;
    a.v_out = (double*)v_out;
    a.chain = 1;
    return psi_fwd_df64(a, st);
  } else if (prec == GPK_FP32) {
    auto a = make_args<float>(T, M, Q, Q, mu0, var0, Z, lls2, lsf2, A, B);
    a.m_out = (float*)m_out;
    a.v_out = (float*)v_out;
    a.chain = 1;
    return psi_fwd_f32(a, st);
  }
  return gpk::fail(GPK_EINVAL, "psi_rollout: unknown precision %d", prec);
}

extern "C" int gpk_psi_bwd_ex(int prec, int N, int M, int Q, int Dout, const void* mu, const void* var,
                              const void* Z, const double* lls2, const double* lsf2, const void* A,
                              const void* B, const void* m, const void* dm, const void* dv, const void* dpsi1,
                              long b_stride, double* dsf2, double* dl, double* dZ, double* dA, double* dB,
                              void* dmu, void* dvar, void* stream);

extern "C" int gpk_psi_bwd(int prec, int N, int M, int Q, int Dout, const void* mu, const void* var,
                           const void* Z, const double* lls2, const double* lsf2, const void* A,
                           const void* B, const void* m, const void* dm, const void* dv, double* dsf2,
                           double* dl, double* dZ, double* dA, double* dB, void* dmu, void* dvar,
                           void* stream) {
  GPK_NVTX("gpk_psi_bwd");
  return gpk_psi_bwd_ex(prec, N, M, Q, Dout, mu, var, Z, lls2, lsf2, A, B, m, dm, dv, nullptr, 0, dsf2, dl, dZ,
                        dA, dB, dmu, dvar, stream);
}

extern "C" int gpk_psi_bwd_ex(int prec, int N, int M, int Q, int Dout, const void* mu, const void* var,
                              const void* Z, const double* lls2, const double* lsf2, const void* A,
                              const void* B, const void* m, const void* dm, const void* dv, const void* dpsi1,
                              long b_stride, double* dsf2, double* dl, double* dZ, double* dA, double* dB,
                              void* dmu, void* dvar, void* stream) {
  GPK_NVTX("gpk_psi_bwd_ex");
  return gpk_psi_bwd_ws(prec, N, M, Q, Dout, mu, var, Z, lls2, lsf2, A, B, m, dm, dv, dpsi1, b_stride, dsf2, dl,
                        dZ, dA, dB, dmu, dvar, nullptr, 0, stream);
}

long psi_bwd_work_elems(int M, int Q, int Dout) {
  const long P = (long)M * (M + 1) / 2;
  return (long)gpk::sm_count() * (Dout * P + (long)Dout * M + (long)M * Q + 1 + Q);
}

extern "C" int gpk_psi_bwd_ws(int prec, int N, int M, int Q, int Dout, const void* mu, const void* var,
                              const void* Z, const double* lls2, const double* lsf2, const void* A,
                              const void* B, const void* m, const void* dm, const void* dv, const void* dpsi1,
                              long b_stride, double* dsf2, double* dl, double* dZ, double* dA, double* dB,
                              void* dmu, void* dvar, double* work, long work_elems, void* stream) {
  GPK_NVTX("gpk_psi_bwd_ws");
  GPK_REQUIRE(N >= 0 && M >= 1 && Q >= 1 && Q <= QMAX, "psi_bwd: bad sizes N=%d M=%d Q=%d", N, M, Q);
  GPK_REQUIRE(Dout >= 1 && Dout <= DMAX, "psi_bwd: Dout=%d outside [1,%d]", Dout, DMAX);
  GPK_REQUIRE(b_stride == 0 || Dout == 1, "psi_bwd: per-point B needs Dout == 1");
  GPK_REQUIRE(mu && var && Z && lls2 && lsf2 && B, "psi_bwd: null input");
  GPK_REQUIRE(dpsi1 || (A && m && dm), "psi_bwd: need dpsi1 or (A, m, dm)");
  GPK_REQUIRE(b_stride != 0 || dv, "psi_bwd: need dv");
  GPK_REQUIRE(dsf2 && dl && dZ && dmu && dvar, "psi_bwd: null output");
  if (work) {
    const long need = psi_bwd_work_elems(M, Q, Dout);
    GPK_REQUIRE(work_elems >= need, "psi_bwd: workspace of %ld doubles, %ld needed", work_elems, need);
  }
  cudaStream_t st = gpk::as_stream(stream);
  const long stride = (long)Dout * M * (M + 1) / 2 + (long)Dout * M + (long)M * Q + 1 + Q;
  if (prec == GPK_DF64) {
    auto a = make_args<double>(N, M, Q, Dout, mu, var, Z, lls2, lsf2, A, B);
    a.m = (const double*)m; a.dm = (const double*)dm; a.dv = (const double*)dv;
    a.dpsi1 = (const double*)dpsi1; a.b_stride = b_stride;
    a.dsf2 = dsf2; a.dl = dl; a.dZ = dZ; a.dA = dA; a.dB = dB;
    a.dmu = (double*)dmu; a.dvar = (double*)dvar;
    a.part = work; a.part_stride = stride;
    return psi_bwd_df64(a, st);
  } else if (prec == GPK_FP32) {
    auto a = make_args<float>(N, M, Q, Dout, mu, var, Z, lls2, lsf2, A, B);
    a.m = (const float*)m; a.dm = (const float*)dm; a.dv = (const float*)dv;
    a.dpsi1 = (const float*)dpsi1; a.b_stride = b_stride;
    a.dsf2 = dsf2; a.dl = dl; a.dZ = dZ; a.dA = dA; a.dB = dB;
    a.dmu = (float*)dmu; a.dvar = (float*)dvar;
    a.part = work; a.part_stride = stride;
    return psi_bwd_f32(a, st);
  }
  return gpk::fail(GPK_EINVAL, "psi_bwd: unknown precision %d", prec);
}

// the translation unit's bounds word (debug build; 0 otherwise)
GPK_BOUNDS_READER(psi_api)
