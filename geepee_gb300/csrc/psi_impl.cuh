// Psi statistics of the ARD kernel under Gaussian inputs, fused with the
// moment-matching contractions of a sparse-GP layer, and their backward pass.
//
// Work decomposition (both kernels): a CTA takes a contiguous range of data points, NPB
// points per pass; per pass its threads first build the points' tables in shared memory
// (per-dimension constants, per-pseudo-input terms u_a, h_aq), then sweep the M(M+1)/2
// unordered pairs (a <= b) of pseudo-inputs, each pair for all NPB points.  Each thread
// owns a fixed set of pairs (p = tid + k*NT) across all of its points, so sums over n of
// per-pair quantities (sum_n psi2, dB = sum_n dv psi2) stay in registers until one atomic
// flush per CTA.  psi2 per point is never materialised in HBM (unless requested).
//
// log psi2[n,a,b] = u_a + u_b + G_ab - sum_q h_aq z_bq   with
//   G_ab = -sum_q (z_aq - z_bq)^2 / (4 l_q)                      (per call, shared memory)
//   u_a  = k_n/2 + sum_q c_q z_aq (mu_q - z_aq/4),  h_aq = c_q z_aq / 2   (per point)
//   k_n  = 2 log sf2 + 1/2 sum_q log(l_q / (l_q + 2 S_q)) - sum_q c_q mu_q^2,
//   c_q  = 1 / (l_q + 2 S_q)
// which is the reference's exponent (geepee/kernels.py:219-225) regrouped so that the
// inner loop costs Q multiply-adds plus one exp.
//
// Template parameters: T compute type (df64 or float); PPT pairs per thread held in
// registers (0: plain strided sweep); QC a compile-time cap on Q and DB on Dout, so
// every per-dimension / per-output array is fully unrolled into registers.
#pragma once
#include "common.cuh"

namespace psi_impl {

constexpr int QMAX = 8;
constexpr int DMAX = 4;
constexpr int NT = 512;        // threads per CTA (forward)
// threads per CTA of the backward (one CTA per SM): 32 warps when Q <= 2 (64 registers a
// thread, no spills), 16 when the per-dimension sums of Q <= 8 need more registers
__host__ __device__ constexpr int nt_bwd(int QC) { return QC <= 2 ? 1024 : 512; }
// Q is QC itself in an exact instantiation (every width other than the two catch-all ones, 2
// for Q <= 2 and QMAX above): the per-dimension loops then carry no runtime test
__host__ __device__ constexpr bool exact_q(int QC) { return QC != 2 && QC != QMAX; }
constexpr int PPT_MAX = 16;    // pairs per thread for register-resident per-pair sums
constexpr int RED = 48;        // reduction slots per warp

template <typename S>
struct PsiArgs {
  int N, M, Q, Dout;
  const S* mu;
  const S* var;
  const S* Z;
  const double* lls2;
  const double* lsf2;
  const S* A;
  const S* B;
  S* psi1;
  S* psi2;
  double* psi2_sum;
  S* m_out;
  S* v_out;
  const S* m;
  const S* dm;
  const S* dv;
  const S* dpsi1;    // optional [N,M]: replaces dm_all A
  int chain;         // forward rollout: point n > 0 takes point n-1's (m, v) as its (mu, var)
  int bs_smem;       // symmetrised B staged in shared memory (set by the launcher)
  int accb_smem;     // backward: dBhat accumulates in shared memory (else atomically in dB)
  int pab_smem;      // backward: the pair table fits in shared memory (set by the launcher)
  long b_stride;     // != 0: B is per point (B + n*b_stride), dv treated as 1
  double* dsf2;
  double* dl;
  double* dZ;
  double* dA;
  double* dB;
  S* dmu;
  S* dvar;
  double* part;      // backward, fixed-order path: this CTA's partial sums at part + blockIdx.x *
                     // part_stride ([dB pairs D*P | dA D*M | dZ M*Q | dsf2 | dl Q]), no atomics
  long part_stride;
};

__device__ __forceinline__ void pair_of(int p, int& a, int& b) { tri_pair(p, a, b); }

// The symmetrised weights of the packed pairs, Bs[d P + p] = B_d[a,b] + B_d[b,a] (a != b) or
// B_d[a,a]: each thread keeps eight pairs' global loads in flight before converting them, so
// the table costs a few memory latencies per CTA instead of one per pair.
template <typename T, int NTH>
__device__ void stage_sym_B(T* Bs, const typename Num<T>::store_t* B, int M, int D, int P) {
  typedef typename Num<T>::store_t S;
  constexpr int K = 8;
  for (int d = 0; d < D; ++d) {
    const S* Bd = B + (size_t)d * M * M;
    for (int p0 = threadIdx.x; p0 < P; p0 += K * NTH) {
      S x1[K], x2[K];
      bool off[K];
#pragma unroll
      for (int k = 0; k < K; ++k) {
        const int p = p0 + k * NTH;
        int ia = 0, ib = 0;
        if (p < P) pair_of(p, ia, ib);
        off[k] = ia != ib;
        x1[k] = p < P ? Bd[ia * M + ib] : S(0);
        x2[k] = off[k] ? Bd[ib * M + ia] : S(0);
      }
#pragma unroll
      for (int k = 0; k < K; ++k) {
        const int p = p0 + k * NTH;
        if (p < P) {
          T w = Num<T>::ld(x1[k]);
          if (off[k]) w = add(w, Num<T>::ld(x2[k]));
          Bs[d * P + p] = w;
        }
      }
    }
  }
}

// CTA-wide sum of K (<= RED) values per thread; the result is valid in warp 0.  Only the
// first `nact` warps hold non-zero values (the others skip the shuffles; default: all).
template <typename T, int K>
__device__ __forceinline__ void block_sum(T* vals, T* red, int nact = 0) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nw = nact > 0 ? nact : (int)(blockDim.x >> 5);
  if (warp < nw) {
#pragma unroll
    for (int i = 0; i < K; ++i) {
      T s = warp_sum(vals[i]);
      if (lane == 0) red[warp * RED + i] = s;
    }
  }
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int i = 0; i < K; ++i) {
      T s = lane < nw ? red[lane * RED + i] : Num<T>::zero();
      vals[i] = warp_sum(s);
    }
  }
}

// block_sum for a point's handful of values: each warp reduces them in multi-value butterflies
// of eight (warp_sum_many; lane 4v then holds value c0 + v), lane i of warp 0 adds value i (and
// i + 32) over the warps in order and shuffles it to the warp.  Fixed order; K <= RED.
template <typename T, int K>
__device__ __forceinline__ void block_sum_many(T (&vals)[K], T* red, int nact) {
  static_assert(K <= RED, "K values per warp slot");
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (warp < nact) {
#pragma unroll
    for (int c0 = 0; c0 < K; c0 += 8) {
      T t[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) t[u] = c0 + u < K ? vals[c0 + u] : Num<T>::zero();
      warp_sum_many<8>(t);
      if ((lane & 3) == 0 && c0 + (lane >> 2) < K) red[warp * RED + c0 + (lane >> 2)] = t[0];
    }
  }
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int c0 = 0; c0 < K; c0 += 32) {
      T s = Num<T>::zero();
      if (c0 + lane < K) {
        s = red[c0 + lane];
        for (int w = 1; w < nact; ++w) s = add(s, red[w * RED + c0 + lane]);
      }
#pragma unroll
      for (int i = c0; i < K && i < c0 + 32; ++i) vals[i] = shfl_idx(s, i - c0);
    }
  }
}

// Per-point tables of one data point n: per-dimension constants (pmu, pis1 = 1/(l+S),
// pc = 1/(l+2S), pld1/pld2 = 1/2 log(l/(l+S)), 1/2 log(l/(l+2S))) and per-pseudo-input terms
// (u_a, h_aq).  The backward keeps one point's tables, the forward NPB points' side by side.
template <typename T>
struct PointSlot {
  T* pmu;
  T* pis1;
  T* pc;
  T* pld1;
  T* pld2;
  T* u;   // [M]
  T* h;   // [M*Q]
};

// per-point constants for dimension q of point n
template <typename T, typename S>
__device__ __forceinline__ void dims_of(const PsiArgs<S>& a, const T* ell2, const T* lnl, const float2* tab,
                                        const PointSlot<T>& ps, int n, int q, int part) {
  // a rollout reads the previous point's outputs (written before the pass's last barrier)
  const S* pmu = a.chain ? (n > 0 ? a.m_out + (size_t)(n - 1) * a.Q : a.mu) : a.mu + (size_t)n * a.Q;
  const S* pvar = a.chain ? (n > 0 ? a.v_out + (size_t)(n - 1) * a.Q : a.var) : a.var + (size_t)n * a.Q;
  // the four transcendental pieces of dimension q run on four threads (part 0..3)
  const T var = Num<T>::ld(pvar[q]);
  const T s = (part & 1) ? add(ell2[q], add(var, var)) : add(ell2[q], var);   // l+2S : l+S
  if (part == 0) {
    ps.pmu[q] = Num<T>::ld(pmu[q]);
    ps.pis1[q] = recip(s);
  } else if (part == 1) {
    ps.pc[q] = recip(s);
  } else if (part == 2) {
    ps.pld1[q] = scale2(sub(lnl[q], log_tab(s, tab)), -1);
  } else {
    ps.pld2[q] = scale2(sub(lnl[q], log_tab(s, tab)), -1);
  }
}

// per-pseudo-input terms of one point: psi1_a (returned), u_a and h_aq (written to the slot)
template <typename T, int QC>
__device__ __forceinline__ T rows_of(const T* z, T lsf, const float2* tab, const PointSlot<T>& ps, int Q, int ia) {
  T e1 = lsf;
  T kap = add(lsf, lsf);
#pragma unroll
  for (int q = 0; q < QC; ++q) {
    if (q < Q) {
      T d = sub(ps.pmu[q], z[ia * Q + q]);
      e1 = add(e1, sub(ps.pld1[q], scale2(mul(mul(d, d), ps.pis1[q]), -1)));
      kap = add(kap, sub(ps.pld2[q], mul(mul(ps.pmu[q], ps.pmu[q]), ps.pc[q])));
    }
  }
  T u = scale2(kap, -1);
#pragma unroll
  for (int q = 0; q < QC; ++q) {
    if (q < Q) {
      T zq = z[ia * Q + q];
      T czq = mul(ps.pc[q], zq);
      u = add(u, mul(czq, sub(ps.pmu[q], scale2(zq, -2))));
      ps.h[ia * Q + q] = scale2(czq, -1);
    }
  }
  ps.u[ia] = u;
  return exp_tab(e1, tab);
}

// ---------------------------------------------------------------------------------
// Forward, NPB points per pass.  Per pass: the NPB points' per-dimension constants (threads
// over (point, q)), then their per-pseudo-input terms (threads over (point, a)), then the pair
// sweep, in which each thread loads a pair's point-independent data once (G_ab, z_b, the
// symmetrised B weights) and evaluates psi2 for all NPB points - NPB independent exp chains
// per pair - and finally one CTA reduction for the NPB points' m and v.  PPT > 0 keeps
// sum_n psi2 of each thread's pairs in registers (pairs tid + k*NT); PPT == 0 sweeps any number
// of pairs.  The pass count, barriers and reductions per point are 1/NPB of a per-point sweep.
template <typename T>
struct FSmem {
  float2* tab;
  T* z;      // [M*Q]
  T* ell2;   // [QMAX]
  T* lnl;    // [QMAX]
  T* inv4l;  // [QMAX]
  T* misc;   // [4] log sf2, sf2
  T* pd;     // [NPB][5][QMAX] per-point constants
  T* u;      // [NPB][M]
  T* h;      // [NPB][M*Q]
  T* p1;     // [NPB][M]
  T* As;     // [Dout][M]
  T* G;      // [P]
  T* Bs;     // [Dout*P] or nullptr
  T* red;    // [32*RED]
};

__host__ __device__ inline size_t fwd_smem_bytes(int M, int Q, int P, int D, int npb, size_t tsz, int nbs) {
  size_t n = (size_t)M * Q + 3 * QMAX + 4 + (size_t)npb * 5 * QMAX + (size_t)npb * M * (2 + Q) + (size_t)D * M + P +
             nbs + 32 * RED;
  return 256 * 8 + n * tsz;
}

template <typename T>
__device__ FSmem<T> fcarve(char* base, int M, int Q, int P, int D, int npb, int nbs) {
  FSmem<T> s;
  s.tab = reinterpret_cast<float2*>(base);
  T* t = reinterpret_cast<T*>(base + 256 * sizeof(float2));
  s.z = t; t += M * Q;
  s.ell2 = t; t += QMAX;
  s.lnl = t; t += QMAX;
  s.inv4l = t; t += QMAX;
  s.misc = t; t += 4;
  s.pd = t; t += npb * 5 * QMAX;
  s.u = t; t += npb * M;
  s.h = t; t += npb * M * Q;
  s.p1 = t; t += npb * M;
  s.As = t; t += D * M;
  s.G = t; t += P;
  s.Bs = nbs ? t : nullptr; t += nbs;
  s.red = t;
  return s;
}

template <typename T>
__device__ __forceinline__ PointSlot<T> fslot(const FSmem<T>& s, int pt, int M, int Q) {
  T* pd = s.pd + pt * 5 * QMAX;
  return PointSlot<T>{pd, pd + QMAX, pd + 2 * QMAX, pd + 3 * QMAX, pd + 4 * QMAX, s.u + pt * M, s.h + pt * M * Q};
}

template <typename T, int NPB, int PPT, int QC, int DB>
__global__ void __launch_bounds__(NT) psi_fwd_kernel(PsiArgs<typename Num<T>::store_t> a) {
  typedef typename Num<T>::store_t S;
  extern __shared__ __align__(16) char smem_raw[];
  const int M = a.M, Q = exact_q(QC) ? QC : a.Q, D = a.Dout;
  const int P = M * (M + 1) / 2;
  const bool contract = (a.A != nullptr) && (a.B != nullptr) && (a.m_out != nullptr || a.v_out != nullptr);
  FSmem<T> s = fcarve<T>(smem_raw, M, Q, P, contract ? D : 0, NPB, a.bs_smem ? D * P : 0);
  // ---- per-CTA tables: exp table, Z, lengthscales, sf2, A, G_ab and the symmetrised B
  load_exp_table(s.tab);
  for (int i = threadIdx.x; i < M * Q; i += NT) s.z[i] = Num<T>::ld(a.Z[i]);
  if (contract)
    for (int i = threadIdx.x; i < D * M; i += NT) s.As[i] = Num<T>::ld(a.A[i]);
  __syncthreads();
  if (threadIdx.x < Q) {
    const int q = threadIdx.x;
    T lnl = Num<T>::ld(static_cast<S>(a.lls2[q]));
    T l2 = exp_tab(lnl, s.tab);
    s.lnl[q] = lnl;
    s.ell2[q] = l2;
    s.inv4l[q] = recip(mul(l2, Num<T>::c(4.f)));
  }
  if (threadIdx.x == 32) {
    T lsf = Num<T>::ld(static_cast<S>(a.lsf2[0]));
    s.misc[0] = lsf;
    s.misc[1] = exp_tab(lsf, s.tab);
  }
  __syncthreads();
  for (int p = threadIdx.x; p < P; p += NT) {
    int ia, ib;
    pair_of(p, ia, ib);
    T g = Num<T>::zero();
#pragma unroll
    for (int q = 0; q < QC; ++q) {
      if (q < Q) {
        T d = sub(s.z[ia * Q + q], s.z[ib * Q + q]);
        g = fma_(mul(d, d), s.inv4l[q], g);
      }
    }
    s.G[p] = neg(g);
  }
  if (s.Bs) stage_sym_B<T, NT>(s.Bs, a.B, M, D, P);
  constexpr int KP = PPT > 0 ? PPT : 1;
  T acc[KP];
  int pab[KP];
#pragma unroll
  for (int k = 0; k < KP; ++k) {
    acc[k] = Num<T>::zero();
    int p = threadIdx.x + k * NT, ia = 0, ib = 0;
    if (PPT > 0 && p < P) pair_of(p, ia, ib);
    pab[k] = (ia << 16) | ib;
  }
  __syncthreads();

  const T lsf = s.misc[0];
  // each CTA takes a contiguous range of points, NPB at a time
  const int nbeg = (int)((long)a.N * blockIdx.x / gridDim.x);
  const int nend = (int)((long)a.N * (blockIdx.x + 1) / gridDim.x);
  for (int n0 = nbeg; n0 < nend; n0 += NPB) {
    const int npts = min(NPB, nend - n0);
    // ---- per-dimension constants of the NPB points
    for (int t = threadIdx.x; t < 4 * npts * Q; t += NT) {
      const int part = t & 3, pq = t >> 2, pt = pq / Q, q = pq - pt * Q;
      dims_of<T, S>(a, s.ell2, s.lnl, s.tab, fslot(s, pt, M, Q), n0 + pt, q, part);
    }
    __syncthreads();
    // ---- per-pseudo-input terms (and psi1)
    for (int t = threadIdx.x; t < npts * M; t += NT) {
      const int pt = t / M, ia = t - pt * M;
      const T v1 = rows_of<T, QC>(s.z, lsf, s.tab, fslot(s, pt, M, Q), Q, ia);
      s.p1[pt * M + ia] = v1;
      if (a.psi1) a.psi1[(size_t)(n0 + pt) * M + ia] = Num<T>::st(v1);
    }
    __syncthreads();
    // ---- pairs
    T vacc[NPB][DB];
#pragma unroll
    for (int pt = 0; pt < NPB; ++pt)
#pragma unroll
      for (int d = 0; d < DB; ++d) vacc[pt][d] = Num<T>::zero();
    auto do_pair = [&](int p, int ia, int ib, T& sum) {
      const T gab = s.G[p];
      T zb[QC];
#pragma unroll
      for (int q = 0; q < QC; ++q) zb[q] = q < Q ? s.z[ib * Q + q] : Num<T>::zero();
      T w[DB];
      if (contract) {
#pragma unroll
        for (int d = 0; d < DB; ++d) {
          w[d] = Num<T>::zero();
          if (d < D) {
            if (s.Bs) {
              w[d] = s.Bs[d * P + p];
            } else {
              const S* Bd = a.B + (size_t)d * M * M;
              w[d] = Num<T>::ld(Bd[ia * M + ib]);
              if (ia != ib) w[d] = add(w[d], Num<T>::ld(Bd[ib * M + ia]));
            }
          }
        }
      }
#pragma unroll
      for (int pt = 0; pt < NPB; ++pt) {
        if (pt < npts) {
          const T* hu = s.u + pt * M;
          const T* hh = s.h + pt * M * Q + ia * Q;
          T x = add(add(hu[ia], hu[ib]), gab);
          T cr = Num<T>::zero();
#pragma unroll
          for (int q = 0; q < QC; ++q)
            if (q < Q) cr = fma_(hh[q], zb[q], cr);
          const T ps = exp_pair(sub(x, cr), s.tab);
          if (a.psi2) {
            const S v = Num<T>::st(ps);
            const size_t o = (size_t)(n0 + pt) * M;
            a.psi2[(o + ia) * M + ib] = v;
            a.psi2[(o + ib) * M + ia] = v;
          }
          if (PPT > 0) sum = add(sum, ps);
          if (contract) {
#pragma unroll
            for (int d = 0; d < DB; ++d)
              if (d < D) vacc[pt][d] = fma_(w[d], ps, vacc[pt][d]);
          }
        }
      }
    };
    // the common configuration (m and v only, Q == QC, Dout == DB, B in shared memory): the same
    // sums without branches, so the NPB points' exps interleave.  In a pass with fewer than NPB
    // points the extra slots run on stale tables; their sums are never read.
    auto do_pair_fast = [&](int p, int ia, int ib) {
      p = GPK_IDX(p, P, 3);
      const T gab = s.G[p];
      T w[DB];
#pragma unroll
      for (int d = 0; d < DB; ++d) w[d] = s.Bs[d * P + p];
      T arg[NPB];
#pragma unroll
      for (int pt = 0; pt < NPB; ++pt) {
        const T* hu = s.u + pt * M;
        const T* hh = s.h + pt * M * QC + ia * QC;
        T cr = mul(hh[0], s.z[ib * QC]);   // = fma_ from zero, bit for bit
#pragma unroll
        for (int q = 1; q < QC; ++q) cr = fma_(hh[q], s.z[ib * QC + q], cr);
        arg[pt] = sub(add(add(hu[ia], hu[ib]), gab), cr);
      }
#pragma unroll
      for (int pt = 0; pt < NPB; ++pt) {
        const T ps = exp_pair(arg[pt], s.tab);
#pragma unroll
        for (int d = 0; d < DB; ++d) vacc[pt][d] = fma_(w[d], ps, vacc[pt][d]);
      }
    };
    const bool fast = PPT == 0 && contract && !a.psi2 && Q == QC && D == DB && s.Bs;
    if (fast) {
      for (int p = threadIdx.x; p < P; p += NT) {
        int ia, ib;
        pair_of(p, ia, ib);
        do_pair_fast(p, ia, ib);
      }
    } else if (PPT > 0) {
#pragma unroll
      for (int k = 0; k < KP; ++k) {
        const int p = threadIdx.x + k * NT;
        if (p < P) do_pair(p, pab[k] >> 16, pab[k] & 0xffff, acc[k]);
      }
    } else {
      T dummy = Num<T>::zero();
      for (int p = threadIdx.x; p < P; p += NT) {
        int ia, ib;
        pair_of(p, ia, ib);
        do_pair(p, ia, ib, dummy);
      }
    }
    if (contract) {
      // m = psi1 . A_d per point, then one CTA reduction of (m, v) for the NPB points
      T vals[2 * NPB * DB];
#pragma unroll
      for (int pt = 0; pt < NPB; ++pt)
#pragma unroll
        for (int d = 0; d < DB; ++d) {
          T mm = Num<T>::zero();
          if (pt < npts && d < D)
            for (int ia = threadIdx.x; ia < M; ia += NT) mm = fma_(s.p1[pt * M + ia], s.As[d * M + ia], mm);
          vals[(pt * DB + d) * 2] = mm;
          vals[(pt * DB + d) * 2 + 1] = vacc[pt][d];
        }
      block_sum_many<T, 2 * NPB * DB>(vals, s.red, NT / 32);
      if (threadIdx.x == 0) {
#pragma unroll
        for (int pt = 0; pt < NPB; ++pt)
#pragma unroll
          for (int d = 0; d < DB; ++d) {
            if (pt < npts && d < D) {
              const int n = n0 + pt;
              const T mm = vals[(pt * DB + d) * 2];
              const T vv = sub(add(s.misc[1], vals[(pt * DB + d) * 2 + 1]), mul(mm, mm));
              if (a.m_out) a.m_out[(size_t)n * D + d] = Num<T>::st(mm);
              if (a.v_out) a.v_out[(size_t)n * D + d] = Num<T>::st(vv);
            }
          }
      }
    }
    __syncthreads();
  }
  if (PPT > 0 && a.psi2_sum) {
#pragma unroll
    for (int k = 0; k < KP; ++k) {
      int p = threadIdx.x + k * NT;
      if (p < P) {
        int ia = pab[k] >> 16, ib = pab[k] & 0xffff;
        double v = (double)Num<T>::st(acc[k]);
        atomicAdd(&a.psi2_sum[ia * M + ib], v);
        if (ia != ib) atomicAdd(&a.psi2_sum[ib * M + ia], v);
      }
    }
  }
}

// ---------------------------------------------------------------------------------
// Backward, NPB points per pass.  Per point: psi1 terms per pseudo-input; per pair
// L = W psi2 with W = sum_d dv_d (B_d[a,b] + B_d[b,a]) (the symmetrised upstream gradient, as
// psi2compDer does, geepee/kernels.py:415-418) staged in shared memory; then per row a the
// full-square sums R_a = sum_b L~_ab, S_aq = sum_b L~_ab z_bq (L~ the symmetric half-weight
// matrix).  Every psi2 gradient is an affine function of R and S:
//   dZ_aq += R_a(-z_aq/l + 2 c mu - c z_aq) + S_aq (1/l - c)
//   dmu_q  = -2c (mu Rt - St)                    (Rt = sum_a R_a, St = sum_a S_a)
//   dS_q   = -c Rt + 2c^2 (mu^2 Rt - 2 mu St + Z2R/2 + ZS/2)
//   dl_q  += 2 ell (Rt (1/(2l) - c/2) + (Z2R - ZS)/(2 l^2) + c^2 (mu^2 Rt - 2 mu St + Z2R/2 + ZS/2))
// with Z2R = sum_a z_a^2 R_a, ZS = sum_a z_a S_a; these restate psi2compDer
// (geepee/kernels.py:402-444) without its N x M x M temporaries.  A pass evaluates each of a
// thread's pairs for all NPB points (the pair's G_ab, z_b and B weights loaded once), and the
// per-point phases and barriers are shared by the NPB points.
template <typename T>
struct BSmem {
  float2* tab;
  T* z;      // [M*Q]
  T* ell2;   // [QMAX]
  T* lnl;    // [QMAX]
  T* inv4l;  // [QMAX]
  T* il;     // [QMAX]
  T* misc;   // [4] log sf2, sf2
  T* pd;     // [NPB][5][QMAX] per-point constants
  T* pg;     // [NPB][2*DMAX] dm_all, dv per point
  T* u;      // [NPB][M]
  T* h;      // [NPB][M*Q]
  T* G;      // [P]
  T* Bs;     // [Dout*P] or nullptr
  T* L;      // [NPB][P]
  T* rows;   // [NPB][M][1+QMAX]
  T* dz;     // [M*Q]
  T* accB;   // [Dout*P] sum over the CTA's points of dv psi2 (dBhat)
  T* red;    // [32*RED]
  int* pab;  // [P] the pairs (a << 16 | b), the same for every point
};

__host__ __device__ inline size_t bwd_smem_bytes(int M, int Q, int P, int nacc, int npb, size_t tsz, int nbs) {
  size_t n = (size_t)M * Q + 4 * QMAX + 4 + (size_t)npb * (5 * QMAX + 2 * DMAX) + (size_t)npb * M * (1 + Q) + P +
             nbs + (size_t)npb * P + (size_t)npb * M * (1 + QMAX) + (size_t)M * Q + nacc + 32 * RED;
  return 256 * 8 + n * tsz;
}

template <typename T>
__device__ BSmem<T> bcarve(char* base, int M, int Q, int P, int nacc, int npb, int nbs) {
  BSmem<T> s;
  s.tab = reinterpret_cast<float2*>(base);
  T* t = reinterpret_cast<T*>(base + 256 * sizeof(float2));
  s.z = t; t += M * Q;
  s.ell2 = t; t += QMAX;
  s.lnl = t; t += QMAX;
  s.inv4l = t; t += QMAX;
  s.il = t; t += QMAX;
  s.misc = t; t += 4;
  s.pd = t; t += npb * 5 * QMAX;
  s.pg = t; t += npb * 2 * DMAX;
  s.u = t; t += npb * M;
  s.h = t; t += npb * M * Q;
  s.G = t; t += P;
  s.Bs = nbs ? t : nullptr; t += nbs;
  s.L = t; t += npb * P;
  s.rows = t; t += npb * M * (1 + QMAX);
  s.dz = t; t += M * Q;
  s.accB = nacc ? t : nullptr; t += nacc;
  s.red = t; t += 32 * RED;
  s.pab = reinterpret_cast<int*>(t);
  return s;
}

template <typename T>
__device__ __forceinline__ PointSlot<T> bslot(const BSmem<T>& s, int pt, int M, int Q) {
  T* pd = s.pd + pt * 5 * QMAX;
  return PointSlot<T>{pd, pd + QMAX, pd + 2 * QMAX, pd + 3 * QMAX, pd + 4 * QMAX, s.u + pt * M, s.h + pt * M * Q};
}

template <typename T, int NPB, int DB, int QC>
__global__ void __launch_bounds__(nt_bwd(QC)) psi_bwd_kernel(PsiArgs<typename Num<T>::store_t> a) {
  constexpr int NTB = nt_bwd(QC);
  typedef typename Num<T>::store_t S;
  extern __shared__ __align__(16) char smem_raw[];
  const int M = a.M, Q = exact_q(QC) ? QC : a.Q, D = a.Dout;
  const int P = M * (M + 1) / 2;
  BSmem<T> s = bcarve<T>(smem_raw, M, Q, P, a.accb_smem ? D * P : 0, NPB, a.bs_smem ? D * P : 0);
  // ---- per-CTA tables: exp table, Z, lengthscales, sf2, G_ab and the symmetrised B
  load_exp_table(s.tab);
  for (int i = threadIdx.x; i < M * Q; i += NTB) {
    s.z[i] = Num<T>::ld(a.Z[i]);
    s.dz[i] = Num<T>::zero();
  }
  if (s.accB)
    for (int i = threadIdx.x; i < D * P; i += NTB) s.accB[i] = Num<T>::zero();
  double* const part = a.part ? a.part + (size_t)blockIdx.x * a.part_stride : nullptr;
  if (part && !s.accB)   // dBhat accumulates in this CTA's partial block (each pair has one owner)
    for (int i = threadIdx.x; i < D * P; i += NTB) part[i] = 0.0;
  __syncthreads();
  if (threadIdx.x < Q) {
    const int q = threadIdx.x;
    T lnl = Num<T>::ld(static_cast<S>(a.lls2[q]));
    T l2 = exp_tab(lnl, s.tab);
    s.lnl[q] = lnl;
    s.ell2[q] = l2;
    s.il[q] = recip(l2);
    s.inv4l[q] = recip(mul(l2, Num<T>::c(4.f)));
  }
  if (threadIdx.x == 32) {
    T lsf = Num<T>::ld(static_cast<S>(a.lsf2[0]));
    s.misc[0] = lsf;
    s.misc[1] = exp_tab(lsf, s.tab);
  }
  __syncthreads();
  for (int p = threadIdx.x; p < P; p += NTB) {
    int ia, ib;
    pair_of(p, ia, ib);
    if (a.pab_smem) s.pab[p] = (ia << 16) | ib;
    T g = Num<T>::zero();
#pragma unroll
    for (int q = 0; q < QC; ++q) {
      if (q < Q) {
        T d = sub(s.z[ia * Q + q], s.z[ib * Q + q]);
        g = fma_(mul(d, d), s.inv4l[q], g);
      }
    }
    s.G[p] = neg(g);
  }
  if (s.Bs) stage_sym_B<T, NTB>(s.Bs, a.B, M, D, P);
  // per-thread accumulators over points
  T g_sf = Num<T>::zero();                 // sum L1 + 2 sum L (for dsf2 * sf2)
  T g_l[QC];                               // dl (before the ell factor)
  T g_A[DB];
#pragma unroll
  for (int q = 0; q < QC; ++q) g_l[q] = Num<T>::zero();
#pragma unroll
  for (int d = 0; d < DB; ++d) g_A[d] = Num<T>::zero();
  const T lsf = s.misc[0];
  __syncthreads();

  // each CTA takes a contiguous range of points, NPB at a time
  const int nbeg = (int)((long)a.N * blockIdx.x / gridDim.x);
  const int nend = (int)((long)a.N * (blockIdx.x + 1) / gridDim.x);
  const int ia0 = threadIdx.x;   // the pseudo-input of this thread in the per-row phases (M <= NTB)
  for (int n0 = nbeg; n0 < nend; n0 += NPB) {
    const int npts = min(NPB, nend - n0);
    // ---- per-point constants and upstream gradients
    for (int t = threadIdx.x; t < 4 * npts * Q; t += NTB) {
      const int part = t & 3, pq = t >> 2, pt = pq / Q, q = pq - pt * Q;
      dims_of<T, S>(a, s.ell2, s.lnl, s.tab, bslot(s, pt, M, Q), n0 + pt, q, part);
    }
    if (threadIdx.x >= 256 && threadIdx.x < 256 + npts * D) {
      const int t = threadIdx.x - 256, pt = t / D, d = t - pt * D, n = n0 + pt;
      T dvv = a.b_stride ? Num<T>::c(1.f) : Num<T>::ld(a.dv[(size_t)n * D + d]);
      if (!a.dpsi1) {
        T mm = Num<T>::ld(a.m[(size_t)n * D + d]);
        T dmv = Num<T>::ld(a.dm[(size_t)n * D + d]);
        s.pg[pt * 2 * DMAX + d] = sub(dmv, mul(scale2(dvv, 1), mm));     // dm_all
      }
      s.pg[pt * 2 * DMAX + DMAX + d] = dvv;
    }
    __syncthreads();
    // ---- psi1 terms, one pseudo-input per thread for all the pass's points
    // vals[pt]: dmu, dS (psi1 part, 2Q) then Rt, St (Q), Z2R (Q), ZS (Q) - reduced together
    constexpr int KV = 5 * QC + 1;
    T vals[NPB * KV];
#pragma unroll
    for (int i = 0; i < NPB * KV; ++i) vals[i] = Num<T>::zero();
    if (ia0 < M) {
#pragma unroll
      for (int pt = 0; pt < NPB; ++pt) {
        if (pt < npts) {
          const int n = n0 + pt;
          const PointSlot<T> ps = bslot(s, pt, M, Q);
          const T* pg = s.pg + pt * 2 * DMAX;
          T p1 = rows_of<T, QC>(s.z, lsf, s.tab, ps, Q, ia0);
          T dp1 = Num<T>::zero();
          if (a.dpsi1) {
            dp1 = Num<T>::ld(a.dpsi1[(size_t)n * M + ia0]);
          } else {
#pragma unroll
            for (int d = 0; d < DB; ++d) {
              if (d < D) {
                dp1 = fma_(pg[d], Num<T>::ld(a.A[d * M + ia0]), dp1);
                g_A[d] = fma_(pg[d], p1, g_A[d]);
              }
            }
          }
          T L1 = mul(dp1, p1);
          g_sf = add(g_sf, L1);
#pragma unroll
          for (int q = 0; q < QC; ++q) {
            if (q < Q) {
              T dd = sub(ps.pmu[q], s.z[ia0 * Q + q]);
              T ds = mul(dd, ps.pis1[q]);                       // (mu - z)/s1
              T ds2 = mul(ds, ds);
              T L1ds = mul(L1, ds);
              vals[pt * KV + q] = neg(L1ds);                    // dmu
              vals[pt * KV + QC + q] = scale2(mul(L1, sub(ds2, ps.pis1[q])), -1);   // dS
              s.dz[ia0 * Q + q] = add(s.dz[ia0 * Q + q], L1ds);  // dZ (psi1)
              g_l[q] = add(g_l[q], mul(L1, add(sub(s.il[q], ps.pis1[q]), ds2)));   // 1/l - 1/s1 + d^2/s1^2
            }
          }
        }
      }
    }
    __syncthreads();
    // ---- pairs: L = W psi2 -> shared memory; dBhat accumulates in shared memory (each
    // pair has one owner thread)
    T dvr[NPB][DB];
#pragma unroll
    for (int pt = 0; pt < NPB; ++pt)
#pragma unroll
      for (int d = 0; d < DB; ++d)
        dvr[pt][d] = (pt < npts && d < D) ? s.pg[pt * 2 * DMAX + DMAX + d] : Num<T>::zero();
    if (NPB == 1 && Q == QC && D == DB && s.Bs && s.accB && !a.b_stride) {
      // the common configuration, branch-free: two pairs (p, p + NTB) per iteration, each step
      // written for both, so that their dependent double-float chains interleave
      const T* hu = s.u;
      for (int p0 = threadIdx.x; p0 < P; p0 += 2 * NTB) {
        int pp[2], ia[2], ib[2];
        bool ok[2];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          ok[u] = p0 + u * NTB < P;
          pp[u] = GPK_IDX(ok[u] ? p0 + u * NTB : p0, P, 2);
          if (a.pab_smem) {   // the pair's (a, b) from the per-CTA table (CTA-uniform test)
            const int ab = s.pab[pp[u]];
            ia[u] = ab >> 16;
            ib[u] = ab & 0xffff;
          } else {
            pair_of(pp[u], ia[u], ib[u]);
          }
        }
        T arg[2];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          const T* hh = s.h + ia[u] * QC;
          T cr = mul(hh[0], s.z[ib[u] * QC]);   // = fma_ from zero, bit for bit
#pragma unroll
          for (int q = 1; q < QC; ++q) cr = fma_(hh[q], s.z[ib[u] * QC + q], cr);
          arg[u] = sub(add(add(hu[ia[u]], hu[ib[u]]), s.G[pp[u]]), cr);
        }
        T ps[2];
#pragma unroll
        for (int u = 0; u < 2; ++u) ps[u] = exp_pair(arg[u], s.tab);
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          T ab[DB];
#pragma unroll
          for (int d = 0; d < DB; ++d) ab[d] = mul(dvr[0][d], ps[u]);
          // L~ (half weight off the diagonal: the symmetric matrix entry) = psi2 sum_d dv_d Bs_d:
          // for one output (dv psi2) Bs, reusing the dB-hat term
          T l;
          if (DB == 1) {
            l = mul(ab[0], s.Bs[pp[u]]);
          } else {
            T w = mul(dvr[0][0], s.Bs[pp[u]]);
#pragma unroll
            for (int d = 1; d < DB; ++d) w = fma_(dvr[0][d], s.Bs[d * P + pp[u]], w);
            l = mul(w, ps[u]);
          }
          if (ok[u]) {
            s.L[pp[u]] = ia[u] == ib[u] ? l : scale2(l, -1);
#pragma unroll
            for (int d = 0; d < DB; ++d) s.accB[d * P + pp[u]] = add(s.accB[d * P + pp[u]], ab[d]);
          }
        }
      }
    } else
    for (int p = threadIdx.x; p < P; p += NTB) {
      int ia, ib;
      pair_of(p, ia, ib);
      const T gab = s.G[p];
      T zb[QC];
#pragma unroll
      for (int q = 0; q < QC; ++q) zb[q] = q < Q ? s.z[ib * Q + q] : Num<T>::zero();
      T bb[DB], ab[DB];
#pragma unroll
      for (int d = 0; d < DB; ++d) {
        bb[d] = ab[d] = Num<T>::zero();
        if (d < D) {
          if (s.Bs) {
            bb[d] = s.Bs[d * P + p];
          } else {
            const S* Bd = a.B + (size_t)d * M * M + (size_t)n0 * a.b_stride;
            bb[d] = Num<T>::ld(Bd[ia * M + ib]);
            if (ia != ib) bb[d] = add(bb[d], Num<T>::ld(Bd[ib * M + ia]));
          }
        }
      }
#pragma unroll
      for (int pt = 0; pt < NPB; ++pt) {
        if (pt < npts) {
          if (a.b_stride && pt > 0) {   // per-point B (Dout == 1): reload for this point
            const S* Bd = a.B + (size_t)(n0 + pt) * a.b_stride;
            bb[0] = Num<T>::ld(Bd[ia * M + ib]);
            if (ia != ib) bb[0] = add(bb[0], Num<T>::ld(Bd[ib * M + ia]));
          }
          const T* hu = s.u + pt * M;
          const T* hh = s.h + pt * M * Q + ia * Q;
          T x = add(add(hu[ia], hu[ib]), gab);
          T cr = Num<T>::zero();
#pragma unroll
          for (int q = 0; q < QC; ++q)
            if (q < Q) cr = fma_(hh[q], zb[q], cr);
          const T ps = exp_pair(sub(x, cr), s.tab);
          T w = Num<T>::zero();
#pragma unroll
          for (int d = 0; d < DB; ++d) {
            if (d < D) {
              w = fma_(dvr[pt][d], bb[d], w);
              ab[d] = fma_(dvr[pt][d], ps, ab[d]);
            }
          }
          // L~ (half weight off the diagonal: the symmetric matrix entry)
          const T l = mul(w, ps);
          s.L[pt * P + p] = ia == ib ? l : scale2(l, -1);
        }
      }
#pragma unroll
      for (int d = 0; d < DB; ++d) {
        if (d < D) {
          if (s.accB) {
            s.accB[d * P + p] = add(s.accB[d * P + p], ab[d]);
          } else if (part) {   // no room for the accumulators: this thread's pair of the partial block
            part[d * P + p] += (double)Num<T>::st(ab[d]);
          } else if (a.dB) {   // no room for the accumulators: straight into dB
            const double v = (double)Num<T>::st(ab[d]);
            atomicAdd(&a.dB[((size_t)d * M + ia) * M + ib], v);
            if (ia != ib) atomicAdd(&a.dB[((size_t)d * M + ib) * M + ia], v);
          }
        }
      }
    }
    __syncthreads();
    // ---- row sums, 8 threads per (point, row)
    for (int rid0 = 0; rid0 < npts * M; rid0 += NTB / 8) {
      const int rid = rid0 + (threadIdx.x >> 3), sl = threadIdx.x & 7;
      const int pt = rid / M, ia = rid - pt * M;
      T R = Num<T>::zero();
      T Sq[QC];
#pragma unroll
      for (int q = 0; q < QC; ++q) Sq[q] = Num<T>::zero();
      if (rid < npts * M) {
        const T* Lp = s.L + pt * P;
        const int rowbase = ia * (ia + 1) / 2;
        // two interleaved partial sums (b = sl + 16 j and sl + 8 + 16 j) halve the chains
        T R1 = Num<T>::zero(), S1[QC];
#pragma unroll
        for (int q = 0; q < QC; ++q) S1[q] = Num<T>::zero();
        // branch-free: a second column past M contributes zero, and dimensions q >= Q reuse
        // dimension 0's coordinate in sums that are never stored
        for (int ib = sl; ib < M; ib += 16) {
          const int jb = ib + 8, jc = jb < M ? jb : ib;
          const int p = ia >= ib ? rowbase + ib : ib * (ib + 1) / 2 + ia;
          const int p1 = ia >= jc ? rowbase + jc : jc * (jc + 1) / 2 + ia;
          const T l = Lp[p];
          const T l1 = jb < M ? Lp[p1] : Num<T>::zero();
          R = add(R, l);
          R1 = add(R1, l1);
#pragma unroll
          for (int q = 0; q < QC; ++q) {
            const int qq = q < Q ? q : 0;
            Sq[q] = fma_(l, s.z[ib * Q + qq], Sq[q]);
            S1[q] = fma_(l1, s.z[jc * Q + qq], S1[q]);
          }
        }
        R = add(R, R1);
#pragma unroll
        for (int q = 0; q < QC; ++q) Sq[q] = add(Sq[q], S1[q]);
      }
#pragma unroll
      for (int m = 1; m < 8; m <<= 1) {
        R = add(R, shfl_xor(R, m));
#pragma unroll
        for (int q = 0; q < QC; ++q) Sq[q] = add(Sq[q], shfl_xor(Sq[q], m));
      }
      if (rid < npts * M && sl == 0) {
        T* row = s.rows + (pt * M + ia) * (1 + QMAX);
        row[0] = R;
#pragma unroll
        for (int q = 0; q < QC; ++q)
          if (q < Q) row[1 + q] = Sq[q];
      }
    }
    __syncthreads();
    // ---- dZ from the row sums, and this row's share of the per-point totals
    if (ia0 < M) {
#pragma unroll
      for (int pt = 0; pt < NPB; ++pt) {
        if (pt < npts) {
          const PointSlot<T> ps = bslot(s, pt, M, Q);
          const T* row = s.rows + (pt * M + ia0) * (1 + QMAX);
          const T R = row[0];
          vals[pt * KV + 2 * QC] = R;
#pragma unroll
          for (int q = 0; q < QC; ++q) {
            if (q < Q) {
              T zq = s.z[ia0 * Q + q];
              T il = s.il[q];
              T cq = ps.pc[q];
              const T Sa = row[1 + q];
              // R(-z/l + 2 c mu - c z) + S (1/l - c)
              T t = sub(add(neg(mul(zq, il)), scale2(mul(cq, ps.pmu[q]), 1)), mul(cq, zq));
              s.dz[ia0 * Q + q] = add(s.dz[ia0 * Q + q], add(mul(R, t), mul(Sa, sub(il, cq))));
              vals[pt * KV + 2 * QC + 1 + q] = Sa;                          // St
              vals[pt * KV + 3 * QC + 1 + q] = mul(mul(zq, zq), R);         // Z2R
              vals[pt * KV + 4 * QC + 1 + q] = mul(zq, Sa);                 // ZS
            }
          }
        }
      }
    }
    // ---- per-point totals: one CTA reduction, then lane q of warp 0 finalises dimension q
    block_sum_many<T, NPB * KV>(vals, s.red, (M + 31) >> 5);   // vals live in the row threads ia0 < M
    if (threadIdx.x < 32) {
#pragma unroll
      for (int pt = 0; pt < NPB; ++pt) {
        if (pt < npts) {
          const int n = n0 + pt;
          const PointSlot<T> ps = bslot(s, pt, M, Q);
          const T Rt = vals[pt * KV + 2 * QC];
#pragma unroll
          for (int q = 0; q < QC; ++q) {
            if (q < Q && q == (int)threadIdx.x) {
              const T St = vals[pt * KV + 2 * QC + 1 + q], Z2R = vals[pt * KV + 3 * QC + 1 + q];
              const T ZS = vals[pt * KV + 4 * QC + 1 + q];
              T mu = ps.pmu[q], cq = ps.pc[q], il = s.il[q];
              T e2 = add(sub(mul(mul(mu, mu), Rt), scale2(mul(mu, St), 1)), scale2(add(Z2R, ZS), -1));
              T dmu = add(vals[pt * KV + q], mul(scale2(cq, 1), sub(St, mul(mu, Rt))));
              T dS = add(vals[pt * KV + QC + q], add(neg(mul(cq, Rt)), scale2(mul(mul(cq, cq), e2), 1)));
              // (dl / 2 ell) accumulates: Rt (1/(2l) - c/2) + (Z2R - ZS)/(2 l^2) + c^2 e2
              T t = add(add(scale2(mul(Rt, sub(il, cq)), -1), scale2(mul(sub(Z2R, ZS), mul(il, il)), -1)),
                        mul(mul(cq, cq), e2));
              g_l[q] = add(g_l[q], scale2(t, 1));
              a.dmu[(size_t)n * Q + q] = Num<T>::st(dmu);
              a.dvar[(size_t)n * Q + q] = Num<T>::st(dS);
            }
          }
          if (threadIdx.x == 0) g_sf = add(g_sf, scale2(Rt, 1));
        }
      }
    }
    __syncthreads();
  }
  // ---- flush CTA accumulators: into the partial block (fixed-order path) or atomically
  T fin[1 + QC];
  fin[0] = g_sf;
#pragma unroll
  for (int q = 0; q < QC; ++q) fin[1 + q] = g_l[q];
  if (part) {
    const bool wantA = a.dA && !a.dpsi1;
    if (s.accB)
      for (int i = threadIdx.x; i < D * P; i += NTB) part[i] = (double)Num<T>::st(s.accB[i]);
    if (threadIdx.x < M) {
#pragma unroll
      for (int d = 0; d < DB; ++d)
        if (d < D) part[D * P + d * M + threadIdx.x] = wantA ? (double)Num<T>::st(g_A[d]) : 0.0;
    }
    for (int i = threadIdx.x; i < M * Q; i += blockDim.x) part[D * P + D * M + i] = (double)Num<T>::st(s.dz[i]);
  } else {
    if (a.dB && s.accB) {
      for (int p = threadIdx.x; p < P; p += NTB) {
        int ia, ib;
        pair_of(p, ia, ib);
        for (int d = 0; d < D; ++d) {
          const double v = (double)Num<T>::st(s.accB[d * P + p]);
          atomicAdd(&a.dB[((size_t)d * M + ia) * M + ib], v);
          if (ia != ib) atomicAdd(&a.dB[((size_t)d * M + ib) * M + ia], v);
        }
      }
    }
    if (threadIdx.x < M) {
#pragma unroll
      for (int d = 0; d < DB; ++d)
        if (d < D && a.dA && !a.dpsi1) atomicAdd(&a.dA[d * M + threadIdx.x], (double)Num<T>::st(g_A[d]));
    }
    for (int i = threadIdx.x; i < M * Q; i += blockDim.x) atomicAdd(&a.dZ[i], (double)Num<T>::st(s.dz[i]));
  }
  // dsf2 and dl need the ell / sf2 factors: (sum L1 + 2 sum L) / sf2 and ell * g_l
  __syncthreads();
  block_sum<T, 1 + QC>(fin, s.red);
  if (threadIdx.x == 0) {
    const double vsf = (double)Num<T>::st(div(fin[0], s.misc[1]));
    if (part) part[D * P + D * M + M * Q] = vsf;
    else atomicAdd(a.dsf2, vsf);
#pragma unroll
    for (int q = 0; q < QC; ++q) {
      if (q < Q) {
        T ell = sqrt_(s.ell2[q]);
        const double vl = (double)Num<T>::st(mul(fin[1 + q], ell));
        if (part) part[D * P + D * M + M * Q + 1 + q] = vl;
        else atomicAdd(&a.dl[q], vl);
      }
    }
  }
}

template <typename T, int NPB, int PPT, int QC, int DB>
int run_fwd(const PsiArgs<typename Num<T>::store_t>& a, int per_sm, size_t sm, cudaStream_t st) {
  auto k = psi_fwd_kernel<T, NPB, PPT, QC, DB>;
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  int resident = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, k, NT, sm);
  if (resident < 1) resident = 1;
  if (resident > per_sm) resident = per_sm;
  int grid = a.chain ? 1 : gpk::sm_count() * resident;   // a rollout is one CTA's sequence
  if (grid > a.N) grid = a.N;
  if (grid < 1) return GPK_OK;
  k<<<grid, NT, sm, st>>>(a);
  return gpk::check_launch("psi_fwd");
}

// points per pass: 4 for Dout <= 2, 2 for Dout <= 4 (so 2*NPB*Dout sums fit one reduction)
template <typename T, int QC>
int fwd_variant(const PsiArgs<typename Num<T>::store_t>& a, bool sum, bool contract, int P, int per_sm, size_t sm,
                cudaStream_t st) {
  if (sum) {
    if (P <= 4 * NT) return run_fwd<T, 2, 4, QC, 4>(a, per_sm, sm, st);
    return run_fwd<T, 2, 16, QC, 4>(a, per_sm, sm, st);
  }
  if (a.chain) {   // one point per pass: each point needs the previous one's moments
    if (a.Dout == 1) return run_fwd<T, 1, 0, QC, 1>(a, per_sm, sm, st);
    if (a.Dout == 2) return run_fwd<T, 1, 0, QC, 2>(a, per_sm, sm, st);
    return run_fwd<T, 1, 0, QC, 4>(a, per_sm, sm, st);
  }
  if (!contract || a.Dout == 1) return run_fwd<T, 4, 0, QC, 1>(a, per_sm, sm, st);
  if (a.Dout == 2) return run_fwd<T, 4, 0, QC, 2>(a, per_sm, sm, st);
  return run_fwd<T, 2, 0, QC, 4>(a, per_sm, sm, st);
}

template <typename T>
int launch_fwd(const PsiArgs<typename Num<T>::store_t>& a_in, cudaStream_t st) {
  PsiArgs<typename Num<T>::store_t> a = a_in;
  const int P = a.M * (a.M + 1) / 2;
  const bool contract = a.A && a.B && (a.m_out || a.v_out);
  const bool sum = a.psi2_sum != nullptr;
  const int npb = a.chain ? 1 : ((sum || (contract && a.Dout > 2)) ? 2 : 4);
  const int D = contract ? a.Dout : 0;
  a.bs_smem = contract && fwd_smem_bytes(a.M, a.Q, P, D, npb, sizeof(T), a.Dout * P) <= 200 * 1024;
  size_t sm = fwd_smem_bytes(a.M, a.Q, P, D, npb, sizeof(T), a.bs_smem ? a.Dout * P : 0);
  if (sm > 227 * 1024) return gpk::fail(GPK_EUNSUPPORTED, "psi_fwd: M=%d needs %zu B of shared memory", a.M, sm);
  if (sum && P > PPT_MAX * NT)
    return gpk::fail(GPK_EUNSUPPORTED, "psi_fwd: psi2_sum needs M(M+1)/2 <= %d (M=%d)", PPT_MAX * NT, a.M);
  int per_sm = (int)((227 * 1024) / (sm + 1024));
  if (per_sm < 1) per_sm = 1;
  if (per_sm > 2) per_sm = 2;
  if (a.Q <= 2) return fwd_variant<T, 2>(a, sum, contract, P, per_sm, sm, st);
  // five input dimensions, one output, moments only (the psi-statistics workload's shape): an
  // exact instantiation, so that the pair loop is the branch-free one (Q == QC)
  if (a.Q == 5 && !sum && !a.chain && contract && a.Dout == 1 && !a.psi2 && a.bs_smem)
    return run_fwd<T, 4, 0, 5, 1>(a, per_sm, sm, st);
  return fwd_variant<T, QMAX>(a, sum, contract, P, per_sm, sm, st);
}

// ---------------------------------------------------------------------------------
// Backward, software-pipelined over points (the common configuration: Q == QC, Dout == DB,
// B and the dB-hat accumulators in shared memory, the fixed-order partial block).  Iteration
// i overlaps point i's front half with point i-1's back half, so a point costs three CTA
// barriers instead of six and the short phases share them:
//   phase 1: row sums of point i-1 (8 threads a row)    | per-point constants of point i
//   phase 2: dZ and totals of point i-1 (warps 4..7)     | psi1 terms of point i (warps 0..3)
//            one CTA reduction of both; warp 0 then finalises point i-1 (dmu, dS)
//   phase 3: the pair sweep of point i (L, dB-hat)
// L, the row sums and the per-pseudo-input tables are read in the phase after the one that
// writes them, so one copy of each suffices; the per-dimension constants, which point i-1's
// finalisation still reads while point i's are formed, alternate between two slots.  The
// psi1 part of a point's dmu, dS waits in shared memory (`carry`) for its finalisation.  The
// arithmetic of every term is psi_bwd_kernel's.
template <typename T>
struct PSmem {
  float2* tab;
  T *z, *ell2, *lnl, *inv4l, *il, *misc;
  T* pd;      // [2][5][QMAX]
  T* pg;      // [2*DMAX] dm_all, dv of the current point
  T* u;       // [M]
  T* h;       // [M*Q]
  T* G;       // [P]
  T* Bs;      // [Dout*P]
  T* L;       // [P]
  T* rows;    // [M][1+QC]
  T* dz;      // [M*Q] psi1 part of dZ
  T* dzr;     // [M*Q] row-sum part of dZ
  T* accB;    // [Dout*P]
  T* carry;   // [2*QC] psi1 part of the previous point's dmu, dS
  T* red;     // [32*RED]
  int* pab;   // [P] the pairs (a << 16 | b), the same for every point
};

__host__ __device__ inline size_t pipe_smem_bytes(int M, int Q, int QC, int P, int D, size_t tsz) {
  const size_t n = (size_t)M * Q + 4 * QMAX + 4 + 2 * 5 * QMAX + 2 * DMAX + M + (size_t)M * Q + P + (size_t)D * P + P +
                   (size_t)M * (1 + QC) + 2 * (size_t)M * Q + (size_t)D * P + 2 * QC + 32 * RED;
  return 256 * 8 + n * tsz + (size_t)P * sizeof(int);
}

template <typename T, int QC>
__device__ PSmem<T> pcarve(char* base, int M, int Q, int P, int D) {
  PSmem<T> s;
  s.tab = reinterpret_cast<float2*>(base);
  T* t = reinterpret_cast<T*>(base + 256 * sizeof(float2));
  s.z = t; t += M * Q;
  s.ell2 = t; t += QMAX;
  s.lnl = t; t += QMAX;
  s.inv4l = t; t += QMAX;
  s.il = t; t += QMAX;
  s.misc = t; t += 4;
  s.pd = t; t += 2 * 5 * QMAX;
  s.pg = t; t += 2 * DMAX;
  s.u = t; t += M;
  s.h = t; t += M * Q;
  s.G = t; t += P;
  s.Bs = t; t += D * P;
  s.L = t; t += P;
  s.rows = t; t += M * (1 + QC);
  s.dz = t; t += M * Q;
  s.dzr = t; t += M * Q;
  s.accB = t; t += D * P;
  s.carry = t; t += 2 * QC;
  s.red = t; t += 32 * RED;
  s.pab = reinterpret_cast<int*>(t);
  return s;
}

template <typename T, int DB, int QC>
__global__ void __launch_bounds__(nt_bwd(QC)) psi_bwd_pipe_kernel(PsiArgs<typename Num<T>::store_t> a) {
  constexpr int NTB = nt_bwd(QC);
  constexpr int Q = QC, D = DB;
  constexpr int KV = 5 * QC + 1;   // [dmu, dS psi1 parts (2QC) | Rt, St (QC), Z2R (QC), ZS (QC)]
  typedef typename Num<T>::store_t S;
  static_assert(NTB >= 8 * 128, "the row phase takes 8 threads for each of up to 128 rows");
  extern __shared__ __align__(16) char smem_raw[];
  const int M = a.M;
  const int P = M * (M + 1) / 2;
  PSmem<T> s = pcarve<T, QC>(smem_raw, M, Q, P, D);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // ---- per-CTA tables (as psi_bwd_kernel)
  load_exp_table(s.tab);
  for (int i = tid; i < M * Q; i += NTB) {
    s.z[i] = Num<T>::ld(a.Z[i]);
    s.dz[i] = Num<T>::zero();
    s.dzr[i] = Num<T>::zero();
  }
  for (int i = tid; i < D * P; i += NTB) s.accB[i] = Num<T>::zero();
  __syncthreads();
  if (tid < Q) {
    const int q = tid;
    T lnl = Num<T>::ld(static_cast<S>(a.lls2[q]));
    T l2 = exp_tab(lnl, s.tab);
    s.lnl[q] = lnl;
    s.ell2[q] = l2;
    s.il[q] = recip(l2);
    s.inv4l[q] = recip(mul(l2, Num<T>::c(4.f)));
  }
  if (tid == 32) {
    T lsf = Num<T>::ld(static_cast<S>(a.lsf2[0]));
    s.misc[0] = lsf;
    s.misc[1] = exp_tab(lsf, s.tab);
  }
  __syncthreads();
  for (int p = tid; p < P; p += NTB) {
    int ia, ib;
    pair_of(p, ia, ib);
    s.pab[p] = (ia << 16) | ib;
    T g = Num<T>::zero();
#pragma unroll
    for (int q = 0; q < QC; ++q) {
      T dd = sub(s.z[ia * Q + q], s.z[ib * Q + q]);
      g = fma_(mul(dd, dd), s.inv4l[q], g);
    }
    s.G[p] = neg(g);
  }
  stage_sym_B<T, NTB>(s.Bs, a.B, M, D, P);
  T g_sf = Num<T>::zero();
  T g_l[QC], g_A[DB];
#pragma unroll
  for (int q = 0; q < QC; ++q) g_l[q] = Num<T>::zero();
#pragma unroll
  for (int d = 0; d < DB; ++d) g_A[d] = Num<T>::zero();
  const T lsf = s.misc[0];
  __syncthreads();

  const int nbeg = (int)((long)a.N * blockIdx.x / gridDim.x);
  const int nend = (int)((long)a.N * (blockIdx.x + 1) / gridDim.x);
  const int cnt = nend - nbeg;
  auto slot = [&](int i) {
    T* pd = s.pd + (i & 1) * 5 * QMAX;
    return PointSlot<T>{pd, pd + QMAX, pd + 2 * QMAX, pd + 3 * QMAX, pd + 4 * QMAX, s.u, s.h};
  };
  for (int i = 0; i <= cnt; ++i) {
    const bool cur = i < cnt, prev = i > 0;
    const int n = nbeg + i;
    // ---- phase 1: row sums of the previous point | constants of this point.  Whole warps
    // enter (the 8-lane sums below shuffle with a full mask); lanes of rows past M add nothing.
    if (prev && warp < (8 * M + 31) / 32) {
      const int ia = tid >> 3, sl = tid & 7;
      const bool live = ia < M;
      T R = Num<T>::zero(), R1 = Num<T>::zero(), Sq[QC], S1[QC];
#pragma unroll
      for (int q = 0; q < QC; ++q) Sq[q] = S1[q] = Num<T>::zero();
      const int rowbase = ia * (ia + 1) / 2;
      for (int ib = sl; live && ib < M; ib += 16) {
        const int jb = ib + 8, jc = jb < M ? jb : ib;
        const int p = ia >= ib ? rowbase + ib : ib * (ib + 1) / 2 + ia;
        const int p1 = ia >= jc ? rowbase + jc : jc * (jc + 1) / 2 + ia;
        const T l = s.L[GPK_IDX(p, P, 6)];
        const T l1 = jb < M ? s.L[GPK_IDX(p1, P, 6)] : Num<T>::zero();
        R = add(R, l);
        R1 = add(R1, l1);
#pragma unroll
        for (int q = 0; q < QC; ++q) {
          Sq[q] = fma_(l, s.z[ib * Q + q], Sq[q]);
          S1[q] = fma_(l1, s.z[jc * Q + q], S1[q]);
        }
      }
      R = add(R, R1);
#pragma unroll
      for (int q = 0; q < QC; ++q) Sq[q] = add(Sq[q], S1[q]);
#pragma unroll
      for (int m = 1; m < 8; m <<= 1) {
        R = add(R, shfl_xor(R, m));
#pragma unroll
        for (int q = 0; q < QC; ++q) Sq[q] = add(Sq[q], shfl_xor(Sq[q], m));
      }
      if (live && sl == 0) {
        T* row = s.rows + ia * (1 + QC);
        row[0] = R;
#pragma unroll
        for (int q = 0; q < QC; ++q) row[1 + q] = Sq[q];
      }
    }
    if (cur) {
      const int t = tid - (NTB - 64);   // the last two warps (beside the row threads while 8 M <= NTB - 64)
      if (t >= 0 && t < 4 * Q) dims_of<T, S>(a, s.ell2, s.lnl, s.tab, slot(i), n, t >> 2, t & 3);
      const int g = tid - (NTB - 32);
      if (g >= 0 && g < D) {
        const T dvv = Num<T>::ld(a.dv[(size_t)n * D + g]);
        const T mm = Num<T>::ld(a.m[(size_t)n * D + g]);
        const T dmv = Num<T>::ld(a.dm[(size_t)n * D + g]);
        s.pg[g] = sub(dmv, mul(scale2(dvv, 1), mm));   // dm_all
        s.pg[DMAX + g] = dvv;
      }
    }
    __syncthreads();
    // ---- phase 2: psi1 terms of this point (warps 0..3) | dZ and totals of the previous (4..7)
    T vals[KV];
#pragma unroll
    for (int k = 0; k < KV; ++k) vals[k] = Num<T>::zero();
    if (cur && tid < M) {
      const int ia0 = tid;
      const PointSlot<T> ps = slot(i);
      const T p1 = rows_of<T, QC>(s.z, lsf, s.tab, ps, Q, ia0);
      T dp1 = Num<T>::zero();
#pragma unroll
      for (int d = 0; d < DB; ++d) {
        dp1 = fma_(s.pg[d], Num<T>::ld(a.A[d * M + ia0]), dp1);
        g_A[d] = fma_(s.pg[d], p1, g_A[d]);
      }
      const T L1 = mul(dp1, p1);
      g_sf = add(g_sf, L1);
#pragma unroll
      for (int q = 0; q < QC; ++q) {
        const T dd = sub(ps.pmu[q], s.z[ia0 * Q + q]);
        const T ds = mul(dd, ps.pis1[q]);
        const T ds2 = mul(ds, ds);
        const T L1ds = mul(L1, ds);
        vals[q] = neg(L1ds);                                            // dmu
        vals[QC + q] = scale2(mul(L1, sub(ds2, ps.pis1[q])), -1);       // dS
        s.dz[ia0 * Q + q] = add(s.dz[ia0 * Q + q], L1ds);               // dZ (psi1)
        g_l[q] = add(g_l[q], mul(L1, add(sub(s.il[q], ps.pis1[q]), ds2)));
      }
    }
    if (prev && tid >= 128 && tid < 128 + M) {
      const int ia0 = tid - 128;
      const PointSlot<T> ps = slot(i - 1);
      const T* row = s.rows + ia0 * (1 + QC);
      const T R = row[0];
      vals[2 * QC] = R;
#pragma unroll
      for (int q = 0; q < QC; ++q) {
        const T zq = s.z[ia0 * Q + q], il = s.il[q], cq = ps.pc[q], Sa = row[1 + q];
        const T t = sub(add(neg(mul(zq, il)), scale2(mul(cq, ps.pmu[q]), 1)), mul(cq, zq));
        s.dzr[ia0 * Q + q] = add(s.dzr[ia0 * Q + q], add(mul(R, t), mul(Sa, sub(il, cq))));
        vals[2 * QC + 1 + q] = Sa;                       // St
        vals[3 * QC + 1 + q] = mul(mul(zq, zq), R);      // Z2R
        vals[4 * QC + 1 + q] = mul(zq, Sa);              // ZS
      }
    }
    block_sum_many<T, KV>(vals, s.red, (128 + M + 31) >> 5);   // warps past the dZ threads hold zeros
    if (warp == 0) {
      if (prev) {   // finalise the previous point with its carried psi1 part
        const int np = n - 1;
        const PointSlot<T> ps = slot(i - 1);
        const T Rt = vals[2 * QC];
#pragma unroll
        for (int q = 0; q < QC; ++q) {
          if (q == lane) {
            const T St = vals[2 * QC + 1 + q], Z2R = vals[3 * QC + 1 + q], ZS = vals[4 * QC + 1 + q];
            const T mu = ps.pmu[q], cq = ps.pc[q], il = s.il[q];
            const T e2 = add(sub(mul(mul(mu, mu), Rt), scale2(mul(mu, St), 1)), scale2(add(Z2R, ZS), -1));
            const T dmu = add(s.carry[q], mul(scale2(cq, 1), sub(St, mul(mu, Rt))));
            const T dS = add(s.carry[QC + q], add(neg(mul(cq, Rt)), scale2(mul(mul(cq, cq), e2), 1)));
            const T t = add(add(scale2(mul(Rt, sub(il, cq)), -1), scale2(mul(sub(Z2R, ZS), mul(il, il)), -1)),
                            mul(mul(cq, cq), e2));
            g_l[q] = add(g_l[q], scale2(t, 1));
            a.dmu[(size_t)np * Q + q] = Num<T>::st(dmu);
            a.dvar[(size_t)np * Q + q] = Num<T>::st(dS);
          }
        }
        if (lane == 0) g_sf = add(g_sf, scale2(Rt, 1));
      }
      __syncwarp();
      if (cur && lane < 2 * QC) s.carry[lane] = vals[lane];   // this point's psi1 part, for its finalisation
    }
    // ---- phase 3: the pair sweep of this point (as psi_bwd_kernel's branch-free loop)
    if (cur) {
      T dvr[DB];
#pragma unroll
      for (int d = 0; d < DB; ++d) dvr[d] = s.pg[DMAX + d];
      for (int p0 = tid; p0 < P; p0 += 2 * NTB) {
        int pp[2], ia[2], ib[2];
        bool ok[2];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          ok[u] = p0 + u * NTB < P;
          pp[u] = ok[u] ? p0 + u * NTB : p0;
          pp[u] = GPK_IDX(pp[u], P, 2);
          const int ab = s.pab[pp[u]];
          ia[u] = ab >> 16;
          ib[u] = ab & 0xffff;
        }
        T arg[2];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          const T* hh = s.h + ia[u] * QC;
          T cr = mul(hh[0], s.z[ib[u] * QC]);   // = fma_ from zero, bit for bit
#pragma unroll
          for (int q = 1; q < QC; ++q) cr = fma_(hh[q], s.z[ib[u] * QC + q], cr);
          arg[u] = sub(add(add(s.u[ia[u]], s.u[ib[u]]), s.G[pp[u]]), cr);
        }
        T ps2[2];
#pragma unroll
        for (int u = 0; u < 2; ++u) ps2[u] = exp_pair(arg[u], s.tab);
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          T ab[DB];
#pragma unroll
          for (int d = 0; d < DB; ++d) ab[d] = mul(dvr[d], ps2[u]);
          // L = psi2 sum_d dv_d Bs_d: for one output (dv psi2) Bs, reusing the dB-hat term
          T l;
          if (DB == 1) {
            l = mul(ab[0], s.Bs[pp[u]]);
          } else {
            T w = mul(dvr[0], s.Bs[pp[u]]);
#pragma unroll
            for (int d = 1; d < DB; ++d) w = fma_(dvr[d], s.Bs[d * P + pp[u]], w);
            l = mul(w, ps2[u]);
          }
          if (ok[u]) {
            s.L[pp[u]] = ia[u] == ib[u] ? l : scale2(l, -1);
#pragma unroll
            for (int d = 0; d < DB; ++d) s.accB[d * P + pp[u]] = add(s.accB[d * P + pp[u]], ab[d]);
          }
        }
      }
    }
    __syncthreads();
  }
  // ---- flush into the partial block: [dB pairs D*P | dA D*M | dZ M*Q | dsf2 | dl Q]
  double* const part = a.part + (size_t)blockIdx.x * a.part_stride;
  for (int i = tid; i < D * P; i += NTB) part[i] = (double)Num<T>::st(s.accB[i]);
  if (tid < M) {
#pragma unroll
    for (int d = 0; d < DB; ++d) part[D * P + d * M + tid] = a.dA ? (double)Num<T>::st(g_A[d]) : 0.0;
  }
  for (int i = tid; i < M * Q; i += NTB) part[D * P + D * M + i] = (double)Num<T>::st(add(s.dz[i], s.dzr[i]));
  T fin[1 + QC];
  fin[0] = g_sf;
#pragma unroll
  for (int q = 0; q < QC; ++q) fin[1 + q] = g_l[q];
  __syncthreads();
  block_sum<T, 1 + QC>(fin, s.red);
  if (tid == 0) {
    part[D * P + D * M + M * Q] = (double)Num<T>::st(div(fin[0], s.misc[1]));
#pragma unroll
    for (int q = 0; q < QC; ++q) part[D * P + D * M + M * Q + 1 + q] = (double)Num<T>::st(mul(fin[1 + q], sqrt_(s.ell2[q])));
  }
}

// the destinations of the backward's partial block (layout in PsiArgs::part)
template <typename S>
gpk::RedPlan bwd_plan(const PsiArgs<S>& a) {
  const int M = a.M, Q = a.Q, D = a.Dout, P = M * (M + 1) / 2;
  gpk::RedPlan r{};
  r.add(a.dB, D * P, 1, M);
  r.add(a.dpsi1 ? nullptr : a.dA, D * M);
  r.add(a.dZ, M * Q);
  r.add(a.dsf2, 1);
  r.add(a.dl, Q);
  return r;
}

template <typename T, int NPB, int DB, int QC>
int run_bwd(const PsiArgs<typename Num<T>::store_t>& a, size_t sm, cudaStream_t st) {
  auto k = psi_bwd_kernel<T, NPB, DB, QC>;
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  int grid = gpk::sm_count();
  if (grid > a.N) grid = a.N;
  if (grid < 1) return GPK_OK;
  k<<<grid, nt_bwd(QC), sm, st>>>(a);
  int rc = gpk::check_launch("psi_bwd");
  if (rc != GPK_OK || !a.part) return rc;
  return gpk::reduce_partials(a.part, grid, bwd_plan(a), st);
}

template <typename T, int DB>
int run_bwd_pipe(const PsiArgs<typename Num<T>::store_t>& a, size_t sm, cudaStream_t st) {
  auto k = psi_bwd_pipe_kernel<T, DB, 2>;
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  int grid = gpk::sm_count();
  if (grid > a.N) grid = a.N;
  if (grid < 1) return GPK_OK;
  k<<<grid, nt_bwd(2), sm, st>>>(a);
  int rc = gpk::check_launch("psi_bwd_pipe");
  if (rc != GPK_OK) return rc;
  return gpk::reduce_partials(a.part, grid, bwd_plan(a), st);
}

template <typename T, int NPB, int QC>
int bwd_db(const PsiArgs<typename Num<T>::store_t>& a, size_t sm, cudaStream_t st) {
  if (a.Dout == 1) return run_bwd<T, NPB, 1, QC>(a, sm, st);
  if (a.Dout == 2) return run_bwd<T, NPB, 2, QC>(a, sm, st);
  return run_bwd<T, NPB, 4, QC>(a, sm, st);
}

// points per pass: BWD_NPB when their tables fit in shared memory and the per-point sums
// (NPB (5 Q + 1) values) fit one reduction; else one
#ifndef GPK_BWD_NPB
#define GPK_BWD_NPB 1
#endif
constexpr int BWD_NPB = GPK_BWD_NPB;
template <typename T>
int launch_bwd(const PsiArgs<typename Num<T>::store_t>& a_in, cudaStream_t st) {
  PsiArgs<typename Num<T>::store_t> a = a_in;
  const int P = a.M * (a.M + 1) / 2;
  if (a.M > nt_bwd(QMAX)) return gpk::fail(GPK_EUNSUPPORTED, "psi_bwd: M=%d > %d", a.M, nt_bwd(QMAX));
  if (5 * (a.Q <= 2 ? 2 : QMAX) + 1 > RED) return gpk::fail(GPK_EUNSUPPORTED, "psi_bwd: Q=%d too large", a.Q);
  const size_t cap = 227 * 1024;
  // the pipelined kernel: Q == 2, Dout <= 2, the fixed-order path, B in shared memory
  if (a.Q == 2 && a.Dout <= 2 && a.part && !a.b_stride && !a.dpsi1 && a.A && a.m && a.dm && a.M <= 128) {
    const size_t sm = pipe_smem_bytes(a.M, 2, 2, P, a.Dout, sizeof(T));
    if (sm <= cap) return a.Dout == 1 ? run_bwd_pipe<T, 1>(a, sm, st) : run_bwd_pipe<T, 2>(a, sm, st);
  }
  const int nbs = a.b_stride == 0 ? a.Dout * P : 0, nacc = a.Dout * P;
  for (int npb = (a.Q <= 2 ? BWD_NPB : 1); npb >= 1; --npb) {
    // preference: B and the dBhat accumulators both in shared memory, then without B, then
    // without either (dBhat then accumulates with atomics in global memory)
    const int opts[3][2] = {{nbs, nacc}, {0, nacc}, {0, 0}};
    for (int o = 0; o < 3; ++o) {
      size_t sm = bwd_smem_bytes(a.M, a.Q, P, opts[o][1], npb, sizeof(T), opts[o][0]);
      if (sm > cap) continue;
      a.bs_smem = opts[o][0] > 0;
      a.accb_smem = opts[o][1] > 0;
      // the pair table only where it fits on top of this option (it never displaces B or the
      // dB-hat accumulators)
      a.pab_smem = sm + (size_t)P * sizeof(int) <= cap;
      if (a.pab_smem) sm += (size_t)P * sizeof(int);
      if (npb == 2) return bwd_db<T, 2, 2>(a, sm, st);
      if (a.Q <= 2) return bwd_db<T, 1, 2>(a, sm, st);
      if (a.Q == 5) return bwd_db<T, 1, 5>(a, sm, st);   // the psi-statistics workload's width, exact
      return bwd_db<T, 1, QMAX>(a, sm, st);
    }
  }
  return gpk::fail(GPK_EUNSUPPORTED, "psi_bwd: M=%d needs too much shared memory", a.M);
}

}  // namespace psi_impl
