// Fused float64 elementwise pieces of the M x M AEP algebra: the q(u) parameter unpacking,
// linear combinations with broadcast, transposes and rank-one terms, the packing of
// d eta1_R, the kernel-hyperparameter chain rule and the natural-parameter log-partition.
// These replace the chains of small tensor operations between the factorisations and the
// products; the arithmetic is plain float64 (the sizes are M^2 per output, so the FP64 pipe
// is not the limit), so every value equals the unfused expression's up to the order of the
// additions.
#include "common.cuh"

namespace {

__global__ void lincomb_kernel(gpk_lincomb_t d) {
  lincomb_run(d, blockIdx.x * (long)blockDim.x + threadIdx.x, (long)gridDim.x * blockDim.x);
}

// R[d] (M x M): upper triangle from the packed eta1_R[d] (row-major triu order), exp() on the
// diagonal, zeros below; lls2 = 2 ls, lsf2 = 2 sf.
__global__ void nat_prep_kernel(int D, int M, int Q, const double* eta1, const double* ls, const double* sf,
                                double* R, double* lls2, double* lsf2) {
  const long total = (long)D * M * M;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
    const int d = (int)(e / ((long)M * M));
    const int r = (int)(e - (long)d * M * M);
    const int a = r / M, b = r - a * M;
    double v = 0.0;
    if (a <= b) {
      const long p = (long)a * M - (long)a * (a - 1) / 2 + (b - a);
      v = eta1[(long)d * M * (M + 1) / 2 + p];
      if (a == b) v = exp(v);
    }
    R[e] = v;
  }
  if (blockIdx.x == 0) {
    for (int q = threadIdx.x; q < Q; q += blockDim.x) lls2[q] = 2.0 * ls[q];
    if (threadIdx.x == 0) lsf2[0] = 2.0 * sf[0];
  }
}

// out[d, p] (+)= dR[d, a, b] * (a == b ? R[d, a, a] : 1) for the upper-triangle entry p = (a, b)
__global__ void triu_pack_kernel(int D, int M, const double* dR, const double* R, double* out, int accumulate) {
  const long total = (long)D * M * M;
  const long P = (long)M * (M + 1) / 2;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
    const int d = (int)(e / ((long)M * M));
    const int r = (int)(e - (long)d * M * M);
    const int a = r / M, b = r - a * M;
    if (a > b) continue;
    const long p = (long)a * M - (long)a * (a - 1) / 2 + (b - a);
    double v = dR[e];
    if (a == b) v *= R[e];
    double* o = out + (long)d * P + p;
    *o = accumulate ? *o + v : v;
  }
}

// g_ls[q] = dl[q] exp(ls[q]);  g_sf = 2 exp(2 sf) (dsf2 + sum(dv))   (one CTA)
__global__ void hyp_grads_kernel(int Q, const double* ls, const double* sf, const double* dl, const double* dsf2,
                                 const double* dv, int ndv, double* g_ls, double* g_sf) {
  __shared__ double red[32];
  double s = 0.0;
  for (int i = threadIdx.x; i < ndv; i += blockDim.x) s += dv[i];
  for (int m = 16; m > 0; m >>= 1) s += __shfl_xor_sync(0xffffffffu, s, m);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    for (int m = 16; m > 0; m >>= 1) s += __shfl_xor_sync(0xffffffffu, s, m);
    if (threadIdx.x == 0) g_sf[0] = 2.0 * exp(2.0 * sf[0]) * (dsf2[0] + s);
  }
  for (int q = threadIdx.x; q < Q; q += blockDim.x) g_ls[q] = dl[q] * exp(ls[q]);
}

// Natural-parameter log-partition of one layer, added into *out with weight w:
//   phi = D/2 logdet Kuu + (N/a - 1)(-1/2 sum logdet Su^-1 + 1/2 mu.th2)
//         - (N/a)(-1/2 sum logdet Suhat^-1 + 1/2 beta muhat.th2)
// (mu.Su^-1 mu = mu.th2 and muhat.Suhat^-1 muhat = beta muhat.th2 because mu = Su th2 and
// muhat = Suhat beta th2.)
__global__ void aep_phi_kernel(int D, int M, double N, double alpha, const double* logdetK,
                               const double* ldSuinv, const double* ldShinv, const double* mu, const double* mh,
                               const double* th2, double w, double* out) {
  __shared__ double red[2][32];
  double qp = 0.0, qc = 0.0;
  for (int i = threadIdx.x; i < D * M; i += blockDim.x) {
    qp += mu[i] * th2[i];
    qc += mh[i] * th2[i];
  }
  for (int m = 16; m > 0; m >>= 1) {
    qp += __shfl_xor_sync(0xffffffffu, qp, m);
    qc += __shfl_xor_sync(0xffffffffu, qc, m);
  }
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = qp;
    red[1][threadIdx.x >> 5] = qc;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    qp = qc = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
      qp += red[0][k];
      qc += red[1][k];
    }
    double lsu = 0.0, lsh = 0.0;
    for (int d = 0; d < D; ++d) {
      lsu -= ldSuinv[d];
      lsh += ldShinv[d];
    }
    const double beta = (N - alpha) / N;
    const double phi = D * 0.5 * logdetK[0] + (N / alpha - 1.0) * (0.5 * lsu + 0.5 * qp) -
                       (N / alpha) * (-0.5 * lsh + 0.5 * beta * qc);
    out[0] += w * phi;
  }
}

// Gaussian likelihood of one minibatch (lik_layers.py:119-181):
//   vt = v + sn2/a, r = y - m;  logZ = sum(-1/2 (log(2 pi vt) + r^2/vt))
//                                     + n D (1/2 log(2 pi sn2/a) - a/2 log(2 pi sn2))
//   dm = scale r/vt,  dv = scale (-1/2/vt + 1/2 r^2/vt^2)
//   energy = scale logZ / N,  g_sn = scale (sum(dv/scale) 2 sn2/a + n D (1 - a)) / N
// Two launches.  gauss_grad_kernel writes dm and dv (the upstream gradients of the whole
// backward) in float64, one division per element, spread over many CTAs (GB300's float64
// units are narrow, so per-element float64 work on one SM is slow).  gauss_sum_kernel (one
// CTA) forms the two sums and the scalars in double-float on the FP32 pipes.
__global__ void __launch_bounds__(128) gauss_grad_kernel(int nD, const double* m, const double* v, const double* y,
                                                         const double* sn, double alpha, double scale, double* dm,
                                                         double* dv) {
  __shared__ double s_sn2a;
  if (threadIdx.x == 0) s_sn2a = exp(2.0 * sn[0]) / alpha;
  __syncthreads();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nD) return;
  const double vt = v[i] + s_sn2a;
  const double r = y[i] - m[i];
  const double ivt = 1.0 / vt;
  const double dmv = r * ivt;
  dm[i] = scale * dmv;
  dv[i] = scale * (0.5 * (r * dmv - 1.0) * ivt);   // -1/(2 vt) + r^2/(2 vt^2)
}

__global__ void __launch_bounds__(1024) gauss_sum_kernel(int n, int D, const double* m, const double* v,
                                                         const double* y, const double* sn, const double* dv,
                                                         double alpha, double scale, double invN, double* energy,
                                                         double* g_sn) {
  __shared__ float2 tab[256];
  __shared__ df64 red[2][32];
  load_exp_table(tab);
  __syncthreads();
  const df64 two_pi = df_from_double(6.283185307179586);
  const df64 sn2 = exp_tab(scale2(df_from_double(sn[0]), 1), tab);
  const df64 sn2a = div(sn2, df_from_double(alpha));
  const df64 inv_scale = recip(df_from_double(scale));
  df64 sl = make_df(0.f), sd = make_df(0.f);
  for (int i = threadIdx.x; i < n * D; i += blockDim.x) {
    const df64 vt = add(df_from_double(v[i]), sn2a);
    const df64 r = sub(df_from_double(y[i]), df_from_double(m[i]));
    sl = add(sl, add(log_tab(mul(two_pi, vt), tab), div(mul(r, r), vt)));
    sd = add(sd, df_from_double(dv[i]));
  }
  sl = warp_sum(sl);
  sd = warp_sum(sd);
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = sl;
    red[1][threadIdx.x >> 5] = sd;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    sl = threadIdx.x < (blockDim.x >> 5) ? red[0][threadIdx.x] : make_df(0.f);
    sd = threadIdx.x < (blockDim.x >> 5) ? red[1][threadIdx.x] : make_df(0.f);
    sl = warp_sum(sl);
    sd = warp_sum(sd);
    if (threadIdx.x == 0) {
      const df64 a_ = df_from_double(alpha);
      const df64 nD = df_from_double((double)n * D);
      const df64 l1 = log_tab(mul(two_pi, sn2a), tab), l2 = log_tab(mul(two_pi, sn2), tab);
      // logZ = -sl/2 + nD (l1/2 - a l2/2)
      const df64 logZ = add(scale2(neg(sl), -1), mul(nD, scale2(sub(l1, mul(a_, l2)), -1)));
      const double sc = scale * invN;
      energy[0] = sc * df_to_double(logZ);
      // sum(dv) / scale * 2 sn2 / a + nD (1 - a)
      const df64 t = add(mul(mul(sd, inv_scale), scale2(sn2a, 1)), mul(nD, sub(make_df(1.f), a_)));
      g_sn[0] = sc * df_to_double(t);
    }
  }
}

// Probit likelihood of binary labels y in {-1, +1} (Probit_Layer.compute_log_Z,
// geepee/lik_layers.py:303-416).  A group of 16 lanes owns one output element e of the
// n x D minibatch.  alpha == 1 takes the closed form: lane s computes sample s,
//   t = y m / sqrt(1 + v),  Z = (1 + erf(t / sqrt 2)) / 2,  logZ = log(Z + eps),
//   dlogZ/dm = phi(t)/(Z + eps) y / sqrt(1 + v),  dlogZ/dv = -phi(t)/(Z + eps) y m / (2 (1 + v)^1.5).
// Otherwise Gauss-Hermite quadrature of the alpha power: lane k takes node k of T <= 16 and
// the group sums over the lanes with shuffles,
//   ts = x_k sqrt(2 v) + m,  p_k = (1 + erf(y ts / sqrt 2)) / 2 + eps,
//   Zt = sum_k w_k p_k^alpha / sqrt(pi),  logZ = log Zt,
//   dZ/dm = sum_k w_k p_k^(alpha-1) exp(-ts^2/2) y alpha / (pi sqrt 2),  dZ/dv = the same with
//   an extra x_k, over sqrt(2 v);  dlogZ/dm = dZ/dm / Zt + eps (and likewise for v).
// The 2-D case (mc = 0, S = 1) uses eps = 1e-8 for the quadrature and 1e-16 for the closed
// form; the sampled 3-D case (mc = 1, m and v [S, n, D]) uses 1e-16 for both and a
// log-mean-exp over the S <= 16 samples, each sample's gradient weighted by its softmax share
// (added eps after the weighting, as the reference does).  The reference's float64 numpy
// expressions are followed operation for operation; erf, exp and log are CUDA's float64
// functions (p^a is exp(a log p)).  dm, dv are written times `scale`; work[e] = the element's
// log-partition for the sum kernel.
__global__ void __launch_bounds__(128) probit_terms_kernel(int S, int nD, int mc, const double* m, const double* v,
                                                           const double* y, double alpha, int T, const double* gh_x,
                                                           const double* gh_w, double scale, double* dm, double* dv,
                                                           double* work) {
  const int lane = threadIdx.x & 15;
  const int e = (int)((blockIdx.x * (long)blockDim.x + threadIdx.x) >> 4);
  if (e >= nD) return;   // whole 16-lane groups leave together
  const unsigned gmask = 0xffffu << (threadIdx.x & 16);
  const double ye = y[e];
  const double kSqrt2 = 1.4142135623730951, kSqrtPi = 1.7724538509055159, kPi = 3.141592653589793;
  double my_lz = -INFINITY, my_dm = 0.0, my_dv = 0.0;
  if (alpha == 1.0) {
    const double eps = 1e-16;
    if (lane < S) {
      const double mm = m[(long)lane * nD + e], vv = v[(long)lane * nD + e];
      const double sv = sqrt(1.0 + vv);
      const double t = ye * mm / sv;
      const double Z = 0.5 * (1.0 + erf(t / kSqrt2));
      my_lz = log(Z + eps);
      const double g = 1.0 / (Z + eps) / sqrt(2.0 * kPi) * exp(-t * t / 2.0);
      my_dm = g * (ye / sv);
      my_dv = g * (-0.5 * ye * mm / ((1.0 + vv) * sv));
    }
  } else {
    const double eps = mc ? 1e-16 : 1e-8;
    const bool node = lane < T;
    const double xk = node ? gh_x[lane] : 0.0, wk = node ? gh_w[lane] : 0.0;
    const double c = ye * alpha / kPi / kSqrt2;
    for (int s = 0; s < S; ++s) {
      const double mm = m[(long)s * nD + e], vv = v[(long)s * nD + e];
      const double s2v = sqrt(2.0 * vv);
      double zt = 0.0, am = 0.0, av = 0.0;
      if (node) {
        const double ts = xk * s2v + mm;
        const double p = 0.5 * (1.0 + erf(ye * ts / kSqrt2)) + eps;
        const double lp = log(p);
        const double pa = exp(alpha * lp);
        const double a = exp((alpha - 1.0) * lp) * exp(-ts * ts / 2.0);
        zt = pa * wk;
        am = wk * a;
        av = wk * (a * xk);
      }
#pragma unroll
      for (int o = 8; o >= 1; o >>= 1) {
        zt += __shfl_xor_sync(gmask, zt, o);
        am += __shfl_xor_sync(gmask, am, o);
        av += __shfl_xor_sync(gmask, av, o);
      }
      zt = zt / kSqrtPi;
      if (lane == s) {
        my_lz = log(zt);
        my_dm = am * c / zt;
        my_dv = av * c / s2v / zt;
      }
    }
  }
  double lse = my_lz, w = 1.0;
  if (mc) {
    double mx = my_lz;
#pragma unroll
    for (int o = 8; o >= 1; o >>= 1) mx = fmax(mx, __shfl_xor_sync(gmask, mx, o));
    const double ex = lane < S ? exp(my_lz - mx) : 0.0;
    double se = ex;
#pragma unroll
    for (int o = 8; o >= 1; o >>= 1) se += __shfl_xor_sync(gmask, se, o);
    lse = mx + log(se) - log((double)S);
    w = ex / se;
  }
  if (lane < S) {
    const double add = alpha == 1.0 ? 0.0 : (mc ? 1e-16 : 1e-8);
    dm[(long)lane * nD + e] = scale * (w * my_dm + add);
    dv[(long)lane * nD + e] = scale * (w * my_dv + add);
  }
  if (lane == 0) work[e] = lse;
}

// Expected log-likelihood under q(f) = N(m, v), the variational free energy's data term.
// kind 0, Gaussian (Gauss_Layer.compute_log_lik_exp and backprop_grads_log_lik_exp,
// geepee/lik_layers.py:183-228), lane 0 of each 16-lane group:
//   q = y^2 - 2 y m + m^2 + v,  ll = -log(2 pi sn2)/2 - q/(2 sn2),  dm = (y - m)/sn2,
//   dv = -1/(2 sn2), and the element's sn term -1 + q/sn2 into work[nD + e].
// kind 1, probit (Probit_Layer.compute_log_lik_exp, lik_layers.py:418-436), lane k = node k:
//   ts = x_k sqrt(2 v) + m, z = y ts,  ll = sum_k w_k/sqrt(pi) log Phi(z),
//   dm = sum_k y w_k/sqrt(pi) phi(z)/Phi(z),  dv = sum_k (the same) x_k sqrt(2/v)/2,
// with Phi(z) = erfc(-z/sqrt 2)/2 and log Phi(z) = log1p(-erfc(z/sqrt 2)/2) for z > 0 (both
// accurate in the tails, as scipy's norm.cdf / norm.logcdf are).  With S > 1 samples (m, v
// [S, n, D] against y [n, D], the 3-D forms) every term is an average over the samples, so each
// element is weighted 1/S.  dm, dv are written times `scale`; work[e] = the element's ll (and,
// Gaussian, work[nSD + e] its sn term), nSD = S n D elements.
__global__ void __launch_bounds__(128) lik_exp_kernel(int kind, int nSD, int nD, const double* m, const double* v,
                                                      const double* y, const double* sn, int T, const double* gh_x,
                                                      const double* gh_w, double scale, double* dm, double* dv,
                                                      double* work) {
  const int lane = threadIdx.x & 15;
  const int e = (int)((blockIdx.x * (long)blockDim.x + threadIdx.x) >> 4);
  if (e >= nSD) return;   // whole 16-lane groups leave together
  const unsigned gmask = 0xffffu << (threadIdx.x & 16);
  const double wS = (double)nD / (double)nSD;   // 1/S
  const double mm = m[e], vv = v[e], ye = y[e % nD];
  const double kSqrt2 = 1.4142135623730951, kSqrtPi = 1.7724538509055159, kPi = 3.141592653589793;
  if (kind == 0) {
    if (lane != 0) return;
    const double sn2 = exp(2.0 * sn[0]);
    const double q = ye * ye - 2.0 * ye * mm + mm * mm + vv;
    work[e] = wS * (-0.5 * log(2.0 * kPi * sn2) - 0.5 / sn2 * q);
    work[nSD + e] = wS * (-1.0 + q / sn2);
    dm[e] = scale * (wS * (1.0 / sn2 * (ye - mm)));
    dv[e] = scale * (wS * (-0.5 / sn2));
    return;
  }
  double ll = 0.0, gm = 0.0, gv = 0.0;
  if (lane < T) {
    const double xk = gh_x[lane], wk = gh_w[lane] / kSqrtPi;
    const double z = (xk * sqrt(2.0 * vv) + mm) * ye;
    const double cdf = 0.5 * erfc(-z / kSqrt2);
    const double lcdf = z > 0.0 ? log1p(-0.5 * erfc(z / kSqrt2)) : log(cdf);
    const double g = ye * wk * (exp(-0.5 * z * z) / sqrt(2.0 * kPi)) / cdf;
    ll = wk * lcdf;
    gm = g;
    gv = g * (0.5 * xk * sqrt(2.0 / vv));
  }
#pragma unroll
  for (int o = 8; o >= 1; o >>= 1) {
    ll += __shfl_xor_sync(gmask, ll, o);
    gm += __shfl_xor_sync(gmask, gm, o);
    gv += __shfl_xor_sync(gmask, gv, o);
  }
  if (lane == 0) {
    work[e] = wS * ll;
    dm[e] = scale * (wS * gm);
    dv[e] = scale * (wS * gv);
  }
}

// out[0] = scale * invN * sum(work[0:nD]) in a fixed order (one CTA).
__global__ void __launch_bounds__(1024) sum_scaled_kernel(int nD, const double* work, double scale, double invN,
                                                          double* out) {
  __shared__ double red[32];
  double s = 0.0;
  for (int i = threadIdx.x; i < nD; i += blockDim.x) s += work[i];
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) out[0] = scale * invN * s;
  }
}

// max |x| over n float64 values as the integer order of their magnitude bits (positive IEEE
// doubles order as their bit patterns), on the integer pipe; the CTA's result in all threads
// max |x_i| over n doubles as the bit pattern of a non-negative double (integer order = value
// order; a NaN's pattern exceeds every finite one), reduced over the CTA.  Four independent
// loads per thread per pass, so that a thread's loads overlap.
__device__ long long maxabs_bits(const double* x, long n, long long* red) {
  constexpr long long MASK = 0x7fffffffffffffffLL;
  long long m0 = 0, m1 = 0, m2 = 0, m3 = 0;
  const long step = blockDim.x;
  long i = threadIdx.x;
  for (; i + 3 * step < n; i += 4 * step) {
    const long long b0 = __double_as_longlong(x[i]) & MASK, b1 = __double_as_longlong(x[i + step]) & MASK;
    const long long b2 = __double_as_longlong(x[i + 2 * step]) & MASK;
    const long long b3 = __double_as_longlong(x[i + 3 * step]) & MASK;
    m0 = b0 > m0 ? b0 : m0;
    m1 = b1 > m1 ? b1 : m1;
    m2 = b2 > m2 ? b2 : m2;
    m3 = b3 > m3 ? b3 : m3;
  }
  for (; i < n; i += step) {
    const long long b = __double_as_longlong(x[i]) & MASK;
    m0 = b > m0 ? b : m0;
  }
  long long m = m0 > m1 ? m0 : m1;
  m2 = m2 > m3 ? m2 : m3;
  m = m > m2 ? m : m2;
  for (int o = 16; o > 0; o >>= 1) {
    const long long v = __shfl_xor_sync(0xffffffffu, m, o);
    m = v > m ? v : m;
  }
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  long long r = 0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) r = red[w] > r ? red[w] : r;
  __syncthreads();
  return r;
}

// one CTA per output d: bit 0 = beta max|T_d| <= max|K^-1|, bit 1 = max|T_d| <= max|K^-1|
constexpr int RG_THREADS = 1024;
__global__ void __launch_bounds__(RG_THREADS) regime_kernel(int M, double beta, const double* T, const double* Kinv,
                                                            int* flags) {
  __shared__ long long red[RG_THREADS / 32];
  const long MM = (long)M * M;
  const double tmax = __longlong_as_double(maxabs_bits(T + blockIdx.x * MM, MM, red));
  const double kmax = __longlong_as_double(maxabs_bits(Kinv, MM, red));
  if (threadIdx.x == 0) flags[blockIdx.x] = (beta * tmax <= kmax ? 1 : 0) | (tmax <= kmax ? 2 : 0);
}

struct FormsArgs {
  int n, chunks;      // items; CTAs per (item, d)
  gpk_forms_t it[GPK_FORMS_MAX];
};

// CTA (c, j): flattened (item, d) = c, element chunk j of that output's M x M block
__global__ void __launch_bounds__(256) cavity_forms_kernel(FormsArgs f) {
  int c = blockIdx.x / f.chunks;
  const int j = blockIdx.x - c * f.chunks;
  int k = 0;
  while (k < f.n && c >= f.it[k].D) c -= f.it[k++].D;
  if (k >= f.n) return;
  const gpk_forms_t& g = f.it[k];
  const int d = c, M = g.M;
  const long MM = (long)M * M;
  const int fl = g.flags[d];
  const bool wc = fl & 1, wp = fl & 2;
  const double b = g.beta;
  const double* T = g.T + d * MM;
  const double *t = g.t + (long)d * M, *vh = g.vh + (long)d * M, *vu = g.vu + (long)d * M;
  if (j == 0) {
    for (int i = threadIdx.x; i < M; i += blockDim.x) {
      g.Ah[(long)d * M + i] = wc ? b * t[i] - b * vh[i] : vh[i];
      g.A[(long)d * M + i] = wp ? t[i] - vu[i] : vu[i];
    }
  }
  const long e0 = MM * j / f.chunks, e1 = MM * (j + 1) / f.chunks;
  const long o = d * MM;
  for (long e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
    const int r = (int)(e / M), q = (int)(e - (long)r * M);
    const double bd = wc ? b * b * g.Qh[o + e] - b * T[e] : g.Qh[o + e] - g.Kinv[e];
    g.Bd[o + e] = bd;
    if (g.Bd_pair) {   // the same value as a double-float pair
      const df64 v = df_from_double(bd);
      reinterpret_cast<float2*>(g.Bd_pair)[o + e] = make_float2(v.hi, v.lo);
    }
    g.Bp[o + e] = wp ? g.Qu[o + e] - T[e] : g.Qu[o + e] - g.Kinv[e];
    const double ar = wc ? b * t[r] - b * vh[r] : vh[r];
    const double aq = wc ? b * t[q] - b * vh[q] : vh[q];
    g.Bsto[o + e] = bd + ar * aq;
    g.G[o + e] = wc ? (r == q ? 1.0 : 0.0) - b * g.Ph[o + e] : g.Ph[o + e];
  }
}

int grid_for(long n) {
  long g = (n + 255) / 256;
  long cap = 4L * gpk::sm_count();
  return (int)(g < 1 ? 1 : (g > cap ? cap : g));
}

}  // namespace

extern "C" int gpk_lincomb(const gpk_lincomb_t* d, void* stream) {
  GPK_NVTX("gpk_lincomb");
  long n = 0;
  if (const int rc = lincomb_check(d, &n)) return rc;
  if (n == 0) return GPK_OK;
  lincomb_kernel<<<grid_for(n), 256, 0, gpk::as_stream(stream)>>>(*d);
  return gpk::check_launch("lincomb");
}

extern "C" int gpk_nat_prep(int D, int M, int Q, const double* eta1, const double* ls, const double* sf, double* R,
                            double* lls2, double* lsf2, void* stream) {
  GPK_NVTX("gpk_nat_prep");
  GPK_REQUIRE(D >= 1 && M >= 1 && Q >= 1, "nat_prep: bad sizes");
  GPK_REQUIRE(eta1 && ls && sf && R && lls2 && lsf2, "nat_prep: null pointer");
  nat_prep_kernel<<<grid_for((long)D * M * M), 256, 0, gpk::as_stream(stream)>>>(D, M, Q, eta1, ls, sf, R, lls2,
                                                                                   lsf2);
  return gpk::check_launch("nat_prep");
}

extern "C" int gpk_triu_pack(int D, int M, const double* dR, const double* R, double* out, int accumulate,
                             void* stream) {
  GPK_NVTX("gpk_triu_pack");
  GPK_REQUIRE(D >= 1 && M >= 1, "triu_pack: bad sizes");
  GPK_REQUIRE(dR && R && out, "triu_pack: null pointer");
  triu_pack_kernel<<<grid_for((long)D * M * M), 256, 0, gpk::as_stream(stream)>>>(D, M, dR, R, out, accumulate);
  return gpk::check_launch("triu_pack");
}

extern "C" int gpk_hyp_grads(int Q, const double* ls, const double* sf, const double* dl, const double* dsf2,
                             const double* dv, int ndv, double* g_ls, double* g_sf, void* stream) {
  GPK_NVTX("gpk_hyp_grads");
  GPK_REQUIRE(Q >= 1 && ndv >= 0, "hyp_grads: bad sizes");
  GPK_REQUIRE(ls && sf && dl && dsf2 && g_ls && g_sf && (dv || ndv == 0), "hyp_grads: null pointer");
  hyp_grads_kernel<<<1, 256, 0, gpk::as_stream(stream)>>>(Q, ls, sf, dl, dsf2, dv, ndv, g_ls, g_sf);
  return gpk::check_launch("hyp_grads");
}

extern "C" int gpk_aep_phi(int D, int M, double N, double alpha, const double* logdetK, const double* ldSuinv,
                           const double* ldShinv, const double* mu, const double* mh, const double* th2, double w,
                           double* out, void* stream) {
  GPK_NVTX("gpk_aep_phi");
  GPK_REQUIRE(D >= 1 && M >= 1 && N > 0 && alpha > 0, "aep_phi: bad sizes");
  GPK_REQUIRE(logdetK && ldSuinv && ldShinv && mu && mh && th2 && out, "aep_phi: null pointer");
  aep_phi_kernel<<<1, 256, 0, gpk::as_stream(stream)>>>(D, M, N, alpha, logdetK, ldSuinv, ldShinv, mu, mh, th2, w,
                                                        out);
  return gpk::check_launch("aep_phi");
}

extern "C" int gpk_gauss_lik(int n, int D, const double* m, const double* v, const double* y, const double* sn,
                             double alpha, double scale, double invN, double* dm, double* dv, double* energy,
                             double* g_sn, int part, void* stream) {
  GPK_NVTX("gpk_gauss_lik");
  GPK_REQUIRE(n >= 0 && D >= 1 && alpha > 0 && scale != 0.0 && part >= 0 && part <= 2, "gauss_lik: bad sizes");
  GPK_REQUIRE(m && v && y && sn && dm && dv && energy && g_sn, "gauss_lik: null pointer");
  cudaStream_t st = gpk::as_stream(stream);
  const int nD = n * D;
  if (part != 2 && nD > 0) gauss_grad_kernel<<<(nD + 127) / 128, 128, 0, st>>>(nD, m, v, y, sn, alpha, scale, dm, dv);
  if (part != 1) gauss_sum_kernel<<<1, 1024, 0, st>>>(n, D, m, v, y, sn, dv, alpha, scale, invN, energy, g_sn);
  return gpk::check_launch("gauss_lik");
}

extern "C" int gpk_probit_lik(int S, int n, int D, int mc, const double* m, const double* v, const double* y,
                              double alpha, int T, const double* gh_x, const double* gh_w, double scale,
                              double invN, double* dm, double* dv, double* work, double* out, void* stream) {
  GPK_NVTX("gpk_probit_lik");
  GPK_REQUIRE(n >= 0 && D >= 1 && S >= 1 && S <= 16 && (mc || S == 1) && alpha > 0 && scale != 0.0,
              "probit_lik: bad sizes");
  GPK_REQUIRE(alpha == 1.0 || (T >= 1 && T <= 16 && gh_x && gh_w), "probit_lik: need 1..16 Gauss-Hermite nodes");
  const long nD = (long)n * D;
  GPK_REQUIRE(out && (nD == 0 || (m && v && y && dm && dv && work)), "probit_lik: null pointer");
  cudaStream_t st = gpk::as_stream(stream);
  GPK_REQUIRE(nD * S < (1L << 31) / 16, "probit_lik: too many elements");
  if (nD > 0) probit_terms_kernel<<<(int)((nD * 16 + 127) / 128), 128, 0, st>>>(S, (int)nD, mc, m, v, y, alpha, T,
                                                                                gh_x, gh_w, scale, dm, dv, work);
  sum_scaled_kernel<<<1, 1024, 0, st>>>((int)nD, work, scale, invN, out);
  return gpk::check_launch("probit_lik");
}

extern "C" int gpk_lik_exp(int kind, int S, int n, int D, const double* m, const double* v, const double* y,
                           const double* sn, int T, const double* gh_x, const double* gh_w, double scale, double invN,
                           double* dm, double* dv, double* work, double* out, double* g_sn, void* stream) {
  GPK_NVTX("gpk_lik_exp");
  GPK_REQUIRE((kind == 0 || kind == 1) && S >= 1 && n >= 0 && D >= 1 && scale != 0.0, "lik_exp: bad sizes");
  GPK_REQUIRE(kind == 0 || (T >= 1 && T <= 16 && gh_x && gh_w), "lik_exp: need 1..16 Gauss-Hermite nodes");
  const long nD = (long)n * D, nSD = nD * S;
  GPK_REQUIRE(nSD < (1L << 31) / 16, "lik_exp: too many elements");
  GPK_REQUIRE(out && (kind == 1 || (sn && g_sn)) && (nD == 0 || (m && v && y && dm && dv && work)),
              "lik_exp: null pointer");
  cudaStream_t st = gpk::as_stream(stream);
  if (nSD > 0) lik_exp_kernel<<<(int)((nSD * 16 + 127) / 128), 128, 0, st>>>(kind, (int)nSD, (int)nD, m, v, y, sn,
                                                                             T, gh_x, gh_w, scale, dm, dv, work);
  sum_scaled_kernel<<<1, 1024, 0, st>>>((int)nSD, work, scale, invN, out);
  if (kind == 0) sum_scaled_kernel<<<1, 1024, 0, st>>>((int)nSD, work + nSD, scale, invN, g_sn);
  return gpk::check_launch("lik_exp");
}

namespace {

// d0[i,:] = s0[idx[i],:] (c0 columns) and d1[i,:] = s1[idx[i],:] (c1 columns) in one pass over
// the n x (c0 + c1) outputs; an index outside [0, rows) gives a NaN row.
__global__ void __launch_bounds__(256) gather_rows_kernel(int n, long long rows, const long long* idx, int c0,
                                                          const double* s0, double* d0, int c1, const double* s1,
                                                          double* d1) {
  const int c = c0 + c1;
  const long long total = (long long)n * c;
  for (long long e = blockIdx.x * 256LL + threadIdx.x; e < total; e += (long long)gridDim.x * 256) {
    const int i = (int)(e / c), j = (int)(e - (long long)i * c);
    const long long r = idx[i];
    const bool ok = r >= 0 && r < rows;
    if (j < c0) d0[(size_t)i * c0 + j] = ok ? s0[(size_t)r * c0 + j] : __longlong_as_double(0x7ff8000000000000LL);
    else d1[(size_t)i * c1 + (j - c0)] = ok ? s1[(size_t)r * c1 + (j - c0)] : __longlong_as_double(0x7ff8000000000000LL);
  }
}

// g[0:span] /= divisor over all CTAs; CTA 0 also writes *worst = max(info[0:ninfo]).
__global__ void __launch_bounds__(256) finish_kernel(int span, double* g, double divisor, int ninfo, const int* info,
                                                     double* worst) {
  for (int i = blockIdx.x * 256 + threadIdx.x; i < span; i += gridDim.x * 256) g[i] /= divisor;
  if (blockIdx.x != 0 || !worst) return;
  __shared__ int wmax[8];
  int v = 0;
  for (int i = threadIdx.x; i < ninfo; i += 256) v = max(v, info[i]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
  if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < 8; ++w) v = max(v, wmax[w]);
    *worst = (double)v;
  }
}

}  // namespace

extern "C" int gpk_gather_rows(int n, long long rows, const long long* idx, int c0, const double* s0, double* d0,
                               int c1, const double* s1, double* d1, void* stream) {
  GPK_NVTX("gpk_gather_rows");
  GPK_REQUIRE(n >= 0 && rows >= 0 && c0 >= 1 && c1 >= 0, "gather_rows: bad sizes n=%d c0=%d c1=%d", n, c0, c1);
  GPK_REQUIRE(idx && s0 && d0 && (c1 == 0 || (s1 && d1)), "gather_rows: null pointer");
  if (n == 0) return GPK_OK;
  const long long total = (long long)n * (c0 + c1);
  const int grid = (int)std::min<long long>((total + 255) / 256, (long long)gpk::sm_count() * 8);
  gather_rows_kernel<<<grid, 256, 0, gpk::as_stream(stream)>>>(n, rows, idx, c0, s0, d0, c1, s1, d1);
  return gpk::check_launch("gather_rows");
}

extern "C" int gpk_finish(int span, double* g, double divisor, int ninfo, const int* info, double* worst,
                          void* stream) {
  GPK_NVTX("gpk_finish");
  GPK_REQUIRE(span >= 0 && ninfo >= 0 && divisor != 0.0, "finish: bad sizes span=%d ninfo=%d", span, ninfo);
  GPK_REQUIRE((span == 0 || g) && (ninfo == 0 || (info && worst)), "finish: null pointer");
  const int grid = std::max(1, std::min((span + 255) / 256, gpk::sm_count()));
  finish_kernel<<<grid, 256, 0, gpk::as_stream(stream)>>>(span, g, divisor, ninfo, ninfo ? info : nullptr,
                                                          ninfo ? worst : nullptr);
  return gpk::check_launch("finish");
}

extern "C" int gpk_regime(int D, int M, double beta, const double* T, const double* Kinv, int* flags,
                          void* stream) {
  GPK_NVTX("gpk_regime");
  GPK_REQUIRE(D >= 1 && D <= 65535 && M >= 1, "regime: bad sizes D=%d M=%d", D, M);
  GPK_REQUIRE(T && Kinv && flags, "regime: null pointer");
  regime_kernel<<<D, RG_THREADS, 0, gpk::as_stream(stream)>>>(M, beta, T, Kinv, flags);
  return gpk::check_launch("regime");
}

extern "C" int gpk_cavity_forms(int n, const gpk_forms_t* items, void* stream) {
  GPK_NVTX("gpk_cavity_forms");
  GPK_REQUIRE(n >= 0 && n <= GPK_FORMS_MAX && (n == 0 || items), "cavity_forms: %d items (max %d)", n, GPK_FORMS_MAX);
  FormsArgs f{};
  f.n = n;
  int total = 0;
  long MM = 0;
  for (int i = 0; i < n; ++i) {
    const gpk_forms_t& g = items[i];
    GPK_REQUIRE(g.D >= 1 && g.M >= 1, "cavity_forms: item %d: bad sizes D=%d M=%d", i, g.D, g.M);
    GPK_REQUIRE(g.T && g.Kinv && g.t && g.Qh && g.Qu && g.vh && g.vu && g.Ph && g.flags && g.Bd && g.Bp && g.Bsto &&
                    g.Ah && g.A && g.G,
                "cavity_forms: item %d: null pointer", i);
    f.it[i] = g;
    total += g.D;
    MM = (long)g.M * g.M > MM ? (long)g.M * g.M : MM;
  }
  if (total == 0) return GPK_OK;
  // 256-element chunks of each output's block, up to about two CTAs per SM in all
  long ch = (MM + 255) / 256;
  const long cap = (2L * gpk::sm_count() + total - 1) / total;
  f.chunks = (int)(ch < 1 ? 1 : (ch > cap ? cap : ch));
  cavity_forms_kernel<<<total * f.chunks, 256, 0, gpk::as_stream(stream)>>>(f);
  return gpk::check_launch("cavity_forms");
}

// the translation unit's bounds word (debug build; 0 otherwise)
GPK_BOUNDS_READER(algebra)
