// Small dense linear algebra for the M x M sparse-GP algebra (M <= 256), double-float.
//   gpk_gemm      batched C = alpha op(A) op(B) + beta C
//   gpk_chol_inv  batched SPD Cholesky + inverse + log-determinant (M <= 128, one CTA each)
//   gpk_trace_kzz gradient of tr(M Kzz) w.r.t. log sf^2, log ell^2 and Z

#include "common.cuh"

namespace {

// An 8-byte element that holds a double-float as its raw (hi, lo) float pair (P2 operands).
template <typename T>
__device__ __forceinline__ T pair_bits(typename Num<T>::store_t v);
template <>
__device__ __forceinline__ df64 pair_bits<df64>(double v) {
  return make_df(__int_as_float(__double2loint(v)), __int_as_float(__double2hiint(v)));
}
template <>
__device__ __forceinline__ float pair_bits<float>(float v) { return v; }

// C tile TBM x TBM per CTA, NG*KS threads: KS groups of NG = (TBM/R)^2 threads each take every
// KS-th k of a chunk (R x R outputs per thread, R = 2 for 32-wide tiles, else 1; 8-wide tiles
// put small products on more SMs), so a thread's chain of dependent
// double-float multiply-adds is k/KS long; the KS partial sums are added through shared
// memory at the end.  The k extent is staged through shared memory in chunks of up to KC,
// and every global load a thread makes for a chunk is issued before any is converted, so a
// chunk costs one memory latency rather than one per element.
constexpr int KC = 128;
// The epilogue is C = alpha acc + beta E, where E may be C itself or another (possibly
// batch-broadcast, sE = 0) matrix.
template <int TBM>
struct GemmShape {
  static constexpr int R = TBM >= 32 ? 2 : 1, TPD = TBM / R, NG = TPD * TPD;
};
template <typename T, int TBM, int KS, bool P2>
__device__ __forceinline__ void gemm_tile(int bx, int by, int bz, int m, int n, int k, int tA, int tB, double alpha,
                                          const typename Num<T>::store_t* A, int lda, long sA,
                                          const typename Num<T>::store_t* B, int ldb, long sB, double beta,
                                          const typename Num<T>::store_t* E, int lde, long sE,
                                          typename Num<T>::store_t* C, int ldc, long sC, double gamma = 0.0,
                                          const typename Num<T>::store_t* U = nullptr, long sU = 0,
                                          const typename Num<T>::store_t* V = nullptr, long sV = 0) {
  typedef typename Num<T>::store_t S;
  constexpr int R = GemmShape<TBM>::R, TPD = GemmShape<TBM>::TPD, NG = GemmShape<TBM>::NG;
  constexpr int NT = NG * KS, NPT = KC * TBM / NT;
  extern __shared__ __align__(16) char smem_raw[];
  T* As = reinterpret_cast<T*>(smem_raw);      // [KC][TBM]
  T* Bs = As + KC * TBM;                        // [KC][TBM]
  A += bz * sA;
  B += bz * sB;
  C += bz * sC;
  if (E) E += bz * sE;
  const int i0 = by * TBM, j0 = bx * TBM;
  const int g = threadIdx.x / NG, t = threadIdx.x % NG;
  const int tx = t % TPD, ty = t / TPD;
  T acc[R][R];
#pragma unroll
  for (int r = 0; r < R; ++r)
#pragma unroll
    for (int c = 0; c < R; ++c) acc[r][c] = Num<T>::zero();
  for (int k0 = 0; k0 < k; k0 += KC) {
    const int kc = min(KC, k - k0);
    // element e < TBM * KC of a tile: (ii, kk) of op(A) / (kk, jj) of op(B), with the
    // compile-time extents TBM and KC as divisors; consecutive threads take consecutive
    // memory, and elements with kk >= kc are skipped
    S ra[NPT], rb[NPT];
    int oa[NPT], ob[NPT];
#pragma unroll
    for (int u = 0; u < NPT; ++u) {
      const int e = threadIdx.x + u * NT;
      ra[u] = rb[u] = S(0);
      oa[u] = ob[u] = -1;
      {
        const int kk = tA ? e / TBM : e % KC, ii = tA ? e % TBM : e / KC;
        if (kk < kc) {
          const int gi = i0 + ii, gk = k0 + kk;
          oa[u] = kk * TBM + ii;
          if (gi < m) ra[u] = tA ? A[(size_t)gk * lda + gi] : A[(size_t)gi * lda + gk];
        }
      }
      {
        const int kk = tB ? e % KC : e / TBM, jj = tB ? e / KC : e % TBM;
        if (kk < kc) {
          const int gj = j0 + jj, gk = k0 + kk;
          ob[u] = kk * TBM + jj;
          if (gj < n) rb[u] = tB ? B[(size_t)gj * ldb + gk] : B[(size_t)gk * ldb + gj];
        }
      }
    }
#pragma unroll
    for (int u = 0; u < NPT; ++u) {
      if (oa[u] >= 0) As[GPK_IDX(oa[u], KC * TBM, 1)] = P2 ? pair_bits<T>(ra[u]) : Num<T>::ld(ra[u]);
      if (ob[u] >= 0) Bs[GPK_IDX(ob[u], KC * TBM, 1)] = P2 ? pair_bits<T>(rb[u]) : Num<T>::ld(rb[u]);
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = g; kk < kc; kk += KS) {
      T av[R], bv[R];
#pragma unroll
      for (int r = 0; r < R; ++r) {
        av[r] = As[kk * TBM + ty * R + r];
        bv[r] = Bs[kk * TBM + tx * R + r];
      }
#pragma unroll
      for (int r = 0; r < R; ++r)
#pragma unroll
        for (int c = 0; c < R; ++c) acc[r][c] = fma_(av[r], bv[c], acc[r][c]);
    }
    __syncthreads();
  }
  if (KS > 1) {
    // the tiles are no longer read (barrier at the end of the last chunk): reuse them
    T* red = As;   // [KS-1][NG][R*R]
    if (g > 0) {
#pragma unroll
      for (int r = 0; r < R; ++r)
#pragma unroll
        for (int c = 0; c < R; ++c) red[((g - 1) * NG + t) * R * R + r * R + c] = acc[r][c];
    }
    __syncthreads();
    if (g > 0) return;
#pragma unroll
    for (int q = 0; q < KS - 1; ++q)
#pragma unroll
      for (int r = 0; r < R; ++r)
#pragma unroll
        for (int c = 0; c < R; ++c) acc[r][c] = add(acc[r][c], red[(q * NG + t) * R * R + r * R + c]);
  }
  // epilogue in the storage type (float64 for df64): the product is rounded once to it, and
  // alpha / beta E enter with that type's arithmetic, as separate BLAS-style operations would
  const S al = static_cast<S>(alpha), be = static_cast<S>(beta), ga = static_cast<S>(gamma);
  if (U) {
    U += bz * sU;
    V += bz * sV;
  }
#pragma unroll
  for (int r = 0; r < R; ++r)
#pragma unroll
    for (int c = 0; c < R; ++c) {
      int gi = i0 + ty * R + r, gj = j0 + tx * R + c;
      if (gi < m && gj < n) {
        S v = Num<T>::st(acc[r][c]);
        if (alpha != 1.0) v = al * v;
        if (beta != 0.0) v = v + be * E[(size_t)gi * lde + gj];
        if (U) v = v + ga * U[gi] * V[gj];   // the rank-one addend
        C[(size_t)gi * ldc + gj] = v;
      }
    }
}

template <typename T, int TBM, int KS, bool P2>
__global__ void __launch_bounds__(GemmShape<TBM>::NG * KS, TBM == 8 ? 6 : 1) gemm_kernel(
    int m, int n, int k, int tA, int tB, double alpha, const typename Num<T>::store_t* A, int lda, long sA,
    const typename Num<T>::store_t* B, int ldb, long sB, double beta, const typename Num<T>::store_t* E, int lde,
    long sE, typename Num<T>::store_t* C, int ldc, long sC) {
  gemm_tile<T, TBM, KS, P2>(blockIdx.x, blockIdx.y, blockIdx.z, m, n, k, tA, tB, alpha, A, lda, sA, B, ldb, sB, beta,
                            E, lde, sE, C, ldc, sC);
}

// Several independent products in one launch: problem p owns the flat tile range
// [first[p], first[p+1]); a CTA finds its problem and runs that tile.
struct GemmGroupArgs {
  int count;
  int first[GPK_GEMM_GROUP + 1];
  int tiles_n[GPK_GEMM_GROUP], tiles_m[GPK_GEMM_GROUP];
  gpk_gemm_t pr[GPK_GEMM_GROUP];
};

// Linear combinations launched with a group of products (one dependency level of the
// algebra): their CTAs follow the products' tiles, descriptor q owning [first[q], first[q+1]).
struct LincombGroupArgs {
  int count;
  int first[GPK_LC_GROUP + 1];
  gpk_lincomb_t d[GPK_LC_GROUP];
};

template <typename T, int TBM, int KS>
__global__ void __launch_bounds__(GemmShape<TBM>::NG * KS, TBM == 8 ? 6 : 1) gemm_group_kernel(GemmGroupArgs g, LincombGroupArgs l) {
  typedef typename Num<T>::store_t S;
  const int ng = g.first[g.count];
  if ((int)blockIdx.x >= ng) {   // a linear-combination CTA (uniform over the CTA)
    const int c = blockIdx.x - ng;
    int q = 0;
#pragma unroll
    for (int u = 1; u < GPK_LC_GROUP; ++u)
      if (u < l.count && c >= l.first[u]) q = u;
    const long nth = blockDim.x;
    lincomb_run(l.d[q], (c - l.first[q]) * nth + threadIdx.x, (long)(l.first[q + 1] - l.first[q]) * nth);
    return;
  }
  const int t = blockIdx.x;
  int p = 0;
#pragma unroll
  for (int q = 1; q < GPK_GEMM_GROUP; ++q)
    if (q < g.count && t >= g.first[q]) p = q;
  const gpk_gemm_t& pr = g.pr[p];
  const int r = t - g.first[p];
  const int per = g.tiles_n[p] * g.tiles_m[p];
  const int bz = r / per, rem = r - bz * per;
  const int by = rem / g.tiles_n[p], bx = rem - by * g.tiles_n[p];
  const void *Ap = pr.A, *Bp = pr.B;
  long sA = pr.strideA, sB = pr.strideB;
  if (pr.sel && ((pr.sel[bz] >> pr.selbit) & 1)) {   // the device-side operand choice (CTA-uniform)
    if (pr.A2) Ap = pr.A2, sA = pr.strideA2;
    if (pr.B2) Bp = pr.B2, sB = pr.strideB2;
  }
  gemm_tile<T, TBM, KS, false>(bx, by, bz, pr.m, pr.n, pr.k, pr.transA, pr.transB, pr.alpha, (const S*)Ap, pr.lda,
                               sA, (const S*)Bp, pr.ldb, sB, pr.beta, (const S*)pr.E, pr.lde, pr.strideE, (S*)pr.C,
                               pr.ldc, pr.strideC, pr.gamma, (const S*)pr.u, pr.strideU, (const S*)pr.v, pr.strideV);
}

// ---- the SPD inverse fast path: factor (one CTA) -> L^-1 (many CTAs) -> L^-T L^-1 (GEMM) ----

// Calls f(std::integral_constant<int, i>) for a warp-uniform runtime i < N, so that register
// arrays are indexed with compile-time constants (no local memory, no select chains).
template <int N, typename F>
__device__ __forceinline__ void with_static(int i, F&& f) {
  if constexpr (N > 0) {
    if (i == N - 1) f(std::integral_constant<int, N - 1>{});
    else with_static<N - 1>(i, f);
  }
}

// f(std::integral_constant<int, I>) for I = 0 .. N-1 in order
template <int I, int N, typename F>
__device__ __forceinline__ void static_for(F&& f) {
  if constexpr (I < N) {
    f(std::integral_constant<int, I>{});
    static_for<I + 1, N>(f);
  }
}

// mbarriers in shared memory (CTA scope): init with an arrival count; arrive (release)
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(bar);
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(a), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(unsigned long long* bar) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(bar);
  asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.shared::cta.b64 st, [%0];\n}\n" ::"r"(a) : "memory");
}
// bounded wait for phase 0 of an mbarrier (acquire): false after ~2^31 SM cycles (about one
// second).  try_wait may suspend the thread until the phase completes, so waiting warps spend
// no issue slots (polling with test_wait measured slower, also for the critical-path warps).
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(bar);
  const long long t0 = clock64();
  do {
    unsigned done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a)
        : "memory");
    if (done) return true;
  } while (clock64() - t0 < (1LL << 31));
  return false;
}

// Two consecutive elements of the pair-interleaved L (one 16-byte load for df64, 8 for FP32)
__device__ __forceinline__ void ld_pair(const df64* p, df64& a, df64& b) {
  const float4 v = *reinterpret_cast<const float4*>(p);
  a = make_df(v.x, v.y);
  b = make_df(v.z, v.w);
}
__device__ __forceinline__ void ld_pair(const float* p, float& a, float& b) {
  const float2 v = *reinterpret_cast<const float2*>(p);
  a = v.x;
  b = v.y;
}

// Right-looking Cholesky of one M x M SPD matrix per CTA (M <= min(32*RS, NW*CS)).  Element
// (i, j) of the lower triangle lives in a register of warp j % NW (column slot j / NW), lane
// (i - j) % 32, row slot (i - j) / 32: each column starts at lane 0 of row slot 0, so a column
// of n rows fills ceil(n / 32) row slots and a trailing update walks only those (a layout
// anchored at row 0 would walk the rows above the diagonal in the same 32-row block and, in
// the last block, the rows past M: 2.3x the element updates of the triangle for M = 100,
// against 1.5x here).  A trailing update touches no shared memory except the columns of L it
// reads.  Column k of L is published by its owner warp through an mbarrier of its own (32
// arrivals); a warp waits only for the columns it applies, so there is no CTA barrier in the
// loop.  Step (k0, k1) = (2s, 2s+1) applies both columns to every column right of k1 (two
// multiply-adds per register slot), so a warp waits, reads its multipliers and walks its
// columns once per two columns.  L is kept in shared memory with the columns of a pair
// interleaved (Lp[s][i][2], s = k / 2), so the two multipliers of a row, and the two
// coefficients of a column, are one load.  Look-ahead: the owner of k2 = k1 + 1 applies the
// pair to that column and publishes it first; the owner of k3 = k2 + 1 applies the pair to
// k3, waits for k2, applies it and publishes k3; then both take their other columns.  The
// look-ahead column's registers are picked by a select chain (runtime slot), so the step is
// one copy of code.  Rows past M in a column's last row slot read the zeroed slack rows of Lp
// and are never stored.  Outputs: Lw (column-major L as raw (hi, lo) pairs, 1/L_kk on the
// diagonal - the input of trinv_kernel), logdet = sum log L_kk^2, info[b] = k+1 for a
// non-positive pivot (M+1 if a bounded wait ran out, never expected).
template <typename T, int RS, int CS, int NW>
__global__ void __launch_bounds__(NW * 32, 1) spd_factor_kernel(int M, const typename Num<T>::store_t* A, long sA,
                                                                 T* Lw, double* logdet, int* info) {
  typedef typename Num<T>::store_t S;
  extern __shared__ __align__(16) char smem_raw[];
  float2* tab = reinterpret_cast<float2*>(smem_raw);
  const int LDP = M + 32;   // rows of a pair (32 slack rows past M)
  const int NP = (M + 1) >> 1;
  T* Lp = reinterpret_cast<T*>(smem_raw + 256 * sizeof(float2));   // [NP][LDP][2]
  T* dg = Lp + (size_t)NP * LDP * 2;                                 // [M] L_kk^2
  T* red = dg + M;                                                   // [NW]
  __shared__ int s_info, s_err;
  __shared__ __align__(8) unsigned long long s_bar[32 * RS];   // column k published (32 arrivals)
  const int b = blockIdx.x, w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  constexpr int NTH = NW * 32;
  static_assert(32 % NW == 0 && NW >= 2 && NW % 2 == 0, "NW must be even and divide 32");
  A += b * sA;
  {
    S* raw = reinterpret_cast<S*>(Lp);   // the staging area (M*M <= NP*LDP*2 elements)
    for (int e = threadIdx.x; e < M * M; e += NTH) {
      const unsigned dst = (unsigned)__cvta_generic_to_shared(raw + e);
      if (sizeof(S) == 8)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(dst), "l"(A + e));
      else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(dst), "l"(A + e));
    }
    asm volatile("cp.async.wait_all;\n" ::);
  }
  load_exp_table(tab);
  if (threadIdx.x == 0) s_info = s_err = 0;
  for (int k = threadIdx.x; k < M; k += NTH) mbar_init(&s_bar[k], 32);
  __syncthreads();
  T a[RS][CS];
  {
    const S* raw = reinterpret_cast<const S*>(Lp);
#pragma unroll
    for (int cc = 0; cc < CS; ++cc)
#pragma unroll
      for (int rr = 0; rr < RS; ++rr) {
        const int j = w + NW * cc, i = j + lane + 32 * rr;
        a[rr][cc] = (i < M) ? Num<T>::ld(raw[i * M + j]) : Num<T>::zero();
      }
  }
  __syncthreads();   // the staging area becomes Lp
  // the slack rows past M of every pair: zeros, read by the rows past M of a last row slot
  for (int e = threadIdx.x; e < NP * 64; e += NTH) Lp[((size_t)(e >> 6) * LDP + M) * 2 + (e & 63)] = Num<T>::zero();
  __syncthreads();
  auto at = [&](int k, int i) -> T* {
    return Lp + GPK_IDX(((size_t)(k >> 1) * LDP + i) * 2 + (k & 1), (size_t)NP * LDP * 2, 0);
  };

  // column k of L from the register column `col` of its owner warp (row k in lane 0, slot 0)
  auto finalize = [&](int k, const T (&col)[RS]) {
    const T p = shfl_idx(col[0], 0);
    if (!(Num<T>::approx(p) > 0.f)) {
      if (lane == 0) s_info = k + 1;
      __syncwarp();
      for (int c = k; c < M; ++c) mbar_arrive(&s_bar[c]);
      return;
    }
    const T r = rsqrt_(p);   // 1 / L_kk
#pragma unroll
    for (int rr = 0; rr < RS; ++rr) {
      const int i = k + lane + 32 * rr;
      if (i > k && i < M) *at(k, i) = mul(col[rr], r);
    }
    if (lane == 0) {
      *at(k, k) = r;
      dg[k] = p;
    }
    __syncwarp();
    mbar_arrive(&s_bar[k]);
  };
  // this thread's register column of slot c (runtime c: a select chain)
  auto column = [&](int c, T (&col)[RS]) {
#pragma unroll
    for (int rr = 0; rr < RS; ++rr) {
      col[rr] = a[rr][0];
#pragma unroll
      for (int cc = 1; cc < CS; ++cc) col[rr] = cc == c ? a[rr][cc] : col[rr];
    }
  };
  // bounded wait for column k; false: stop (a wait ran out, or a pivot failed)
  auto await = [&](int k) {
    if (!mbar_wait(&s_bar[k])) {
      if (lane == 0) s_err = 1;
      return false;
    }
    return s_info == 0;
  };
  // the pair (k0, k0 + 1) applied to the rows of column j held in v (row slots below nr)
  auto apply_pair = [&](int k0, int j, int nr, T* v) {
    T x0, x1;
    ld_pair(at(k0, j), x0, x1);
#pragma unroll
    for (int rr = 0; rr < RS; ++rr) {
      if (rr > 0 && rr >= nr) break;   // warp-uniform
      T l0, l1;
      ld_pair(at(k0, j + lane + 32 * rr), l0, l1);
      v[rr] = fma_(neg(l1), x1, fma_(neg(l0), x0, v[rr]));
    }
  };

  // columns 0 and 1 before the first step
  if (w == 0) {
    T col[RS];
    column(0, col);
    finalize(0, col);
  }
  if (w == 1 && M > 1) {
    if (await(0)) {
      T col[RS];
      column(0, col);
      const T x = *at(0, 1);
      const int nr = (M - 1 + 31) >> 5;
#pragma unroll
      for (int rr = 0; rr < RS; ++rr)
        if (rr < nr) col[rr] = fma_(neg(*at(0, 1 + lane + 32 * rr)), x, col[rr]);
      finalize(1, col);
    }
  }
  const int ncol = w < M ? (M - 1 - w) / NW + 1 : 0;   // this warp's columns
  const int last = w + NW * (ncol - 1);
  bool stop = ncol == 0;
  for (int k2 = 2; !stop; k2 += 2) {
    const int k3 = k2 + 1, k0 = k2 - 2, k1 = k2 - 1;
    if (k1 >= M - 1 || last <= k1) break;   // nothing of this warp right of the pair
    if (!await(k1)) break;                  // k1 published implies k0 published
    const int C = k2 / NW;                  // the look-ahead pair's slot in its owners
    const bool own2 = w == k2 % NW, own3 = w == k3 % NW && k3 < M;
    if (own2 || own3) {   // look-ahead: column k2, or column k3 (which also needs column k2)
      const int kx = own2 ? k2 : k3;
      const int nr = (M - kx + 31) >> 5;
      T col[RS];
      column(C, col);
      apply_pair(k0, kx, nr, col);
      if (own3) {
        if (!await(k2)) break;
        const T x2 = *at(k2, k3);
#pragma unroll
        for (int rr = 0; rr < RS; ++rr) {
          if (rr > 0 && rr >= nr) break;
          col[rr] = fma_(neg(*at(k2, k3 + lane + 32 * rr)), x2, col[rr]);
        }
      }
      finalize(kx, col);   // the register column is dead afterwards
    }
    // the pair on every other column of this warp right of k1
    const int clo = k1 >= w ? (k1 - w) / NW + 1 : 0;   // first slot with column > k1
#pragma unroll
    for (int cc = 0; cc < CS; ++cc) {
      if (cc < clo || cc >= ncol || ((own2 || own3) && cc == C)) continue;   // warp-uniform
      const int j = w + NW * cc;
      const int nr = (M - j + 31) >> 5;
      T x0, x1;
      ld_pair(at(k0, j), x0, x1);
      // row slots past (32*RS - NW*cc) / 32 hold no row of any column of this slot
#pragma unroll
      for (int rr = 0; rr < RS - ((NW * cc) >> 5); ++rr) {
        if (rr > 0 && rr >= nr) break;   // warp-uniform
        T l0, l1;
        ld_pair(at(k0, j + lane + 32 * rr), l0, l1);
        a[rr][cc] = fma_(neg(l1), x1, fma_(neg(l0), x0, a[rr][cc]));
      }
    }
  }
  __syncthreads();
  if (threadIdx.x == 0 && s_err && !s_info) s_info = M + 1;
  __syncthreads();
  const int bad = s_info;
  if (info && threadIdx.x == 0) info[b] = bad;
  if (bad) return;
  T* Lb = Lw + (size_t)b * M * M;
  for (int e = threadIdx.x; e < M * M; e += NTH) {
    const int k = e / M, i = e - k * M;
    if (i >= k) Lb[e] = *at(k, i);
  }
  if (logdet) {
    T l = Num<T>::zero();
    for (int i = threadIdx.x; i < M; i += NTH) l = add(l, log_tab(dg[i], tab));
    l = warp_sum(l);
    if (lane == 0) red[w] = l;
    __syncthreads();
    if (w == 0) {
      T s2 = warp_sum(lane < NW ? red[lane] : Num<T>::zero());
      if (lane == 0) logdet[b] = (double)Num<T>::st(s2);
    }
  }
}

// X = L^-1 by columns: warp j solves L x = e_j by right-looking forward substitution
//   x_k = t_k / L_kk,  t_i -= L_ik x_k (i > k),  t = e_j at start,
// with row k held by lane k % 32 and broadcast by shuffle; columns are independent, so the
// CTAs of a launch (TW columns each) run side by side.  Input: Lw from spd_factor_kernel
// (column-major, 1/L_kk on the diagonal); output Xt[b][j*M + i] = X_ij (i.e. X^T row-major,
// zeros for i < j).  info[b] != 0 (a failed factorisation) leaves Xt untouched.
constexpr int TW = 4;
template <typename T, int RS>
__global__ void __launch_bounds__(TW * 32) trinv_kernel(int M, const T* Lw, T* Xt, const int* info) {
  extern __shared__ __align__(16) char smem_raw[];
  const int b = blockIdx.y;
  if (info && info[b]) return;
  const int j0 = blockIdx.x * TW;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // columns k >= j0 of L (rows >= k) into shared memory: Ls[(k - j0) * M + i]
  T* Ls = reinterpret_cast<T*>(smem_raw);
  const T* Lb = Lw + (size_t)b * M * M + (size_t)j0 * M;
  const int n = (M - j0) * M;
  for (int e = threadIdx.x; e < n; e += TW * 32) {
    const unsigned dst = (unsigned)__cvta_generic_to_shared(Ls + e);
    if (sizeof(T) == 8)
      asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(dst), "l"(Lb + e));
    else
      asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(dst), "l"(Lb + e));
  }
  asm volatile("cp.async.wait_all;\n" ::);
  __syncthreads();
  const int j = j0 + w;
  if (j >= M) return;
  T t[RS];
#pragma unroll
  for (int rr = 0; rr < RS; ++rr) t[rr] = (lane + 32 * rr == j) ? Num<T>::c(1.f) : Num<T>::zero();
  // k = 32 kb + kk: the slot kb of the pivot row is a compile-time index (no selects or
  // branches on the loop-carried path), the pivot lane is kk
  const int kb0 = j >> 5;
#pragma unroll
  for (int kb = 0; kb < RS; ++kb) {
    if (kb < kb0) continue;   // warp-uniform
    const int kend = min(32, M - 32 * kb);
    for (int kk = (kb == kb0 ? (j & 31) : 0); kk < kend; ++kk) {
      const int k = 32 * kb + kk;
      const T* col = Ls + (size_t)(k - j0) * M;
      const T xk = mul(shfl_idx(t[kb], kk), col[k]);
      t[kb] = lane == kk ? xk : t[kb];
#pragma unroll
      for (int rr = kb; rr < RS; ++rr) {
        const int i = lane + 32 * rr;
        const T lik = col[min(i, M - 1)];
        t[rr] = fma_(neg(i > k && i < M ? lik : Num<T>::zero()), xk, t[rr]);
      }
    }
  }
  T* Xb = Xt + (size_t)b * M * M + (size_t)j * M;
#pragma unroll
  for (int rr = 0; rr < RS; ++rr) {
    const int i = lane + 32 * rr;
    if (i < M) Xb[i] = i >= j ? t[rr] : Num<T>::zero();
  }
}

// GMEM = false: the matrix lives in shared memory (M <= 128).  GMEM = true: it lives in the
// caller's workspace (work, M*M elements per matrix, L2-resident), any M.
template <typename T, bool GMEM>
__global__ void __launch_bounds__(1024) chol_inv_kernel(int M, const typename Num<T>::store_t* A, long sA,
                                                        typename Num<T>::store_t* Ainv, long sI,
                                                        typename Num<T>::store_t* Lout, long sL, double* logdet,
                                                        int* info, typename Num<T>::store_t* work,
                                                        typename Num<T>::store_t* Xout) {
  extern __shared__ __align__(16) char smem_raw[];
  float2* tab = reinterpret_cast<float2*>(smem_raw);
  const int b = blockIdx.x;
  const int ld = GMEM ? M : M + 1;
  T* base = reinterpret_cast<T*>(smem_raw + 256 * sizeof(float2));
  T* S = GMEM ? reinterpret_cast<T*>(work) + (size_t)b * M * M : base;   // [M][ld]
  T* dg = GMEM ? base : base + M * ld;                             // [M] diagonal of L
  T* di = dg + M;                                                  // [M] 1/diag
  T* tmp = di + M;                                                 // [M]
  T* red = tmp + M;                                                // [32]
  __shared__ int s_info;
  A += b * sA;
  const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;
  load_exp_table(tab);
  for (int e = tid; e < M * M; e += blockDim.x) {
    int i = e / M, j = e % M;
    S[i * ld + j] = Num<T>::ld(A[(size_t)i * M + j]);
  }
  if (tid == 0) s_info = 0;
  __syncthreads();
  // right-looking Cholesky on the lower triangle.  The square root and reciprocal of each
  // pivot are computed once, by the thread that finalises that diagonal entry in the
  // previous step's trailing update, and published through shared memory.
  if (tid == 0) {
    T piv = S[0];
    if (!(Num<T>::approx(piv) > 0.f)) {
      s_info = 1;
    } else {
      T d = sqrt_(piv);
      dg[0] = d;
      di[0] = recip(d);
    }
  }
  __syncthreads();
  for (int kk = 0; kk < M; ++kk) {
    if (s_info) break;   // uniform: written before the last barrier
    const T inv = di[kk];
    for (int i = kk + 1 + tid; i < M; i += blockDim.x) S[i * ld + kk] = mul(S[i * ld + kk], inv);
    __syncthreads();
    for (int i = kk + 1 + ty; i < M; i += 32) {
      T lik = S[i * ld + kk];
      for (int j = kk + 1 + tx; j <= i; j += 32) {
        T v = sub(S[i * ld + j], mul(lik, S[j * ld + kk]));
        S[i * ld + j] = v;
        if (i == kk + 1 && j == kk + 1) {
          if (!(Num<T>::approx(v) > 0.f)) {
            s_info = kk + 2;
          } else {
            T d = sqrt_(v);
            dg[kk + 1] = d;
            di[kk + 1] = recip(d);
          }
        }
      }
    }
    __syncthreads();
  }
  int bad = s_info;
  if (info && tid == 0) info[b] = bad;
  if (bad) return;
  if (Lout) {
    Lout += b * sL;
    for (int e = tid; e < M * M; e += blockDim.x) {
      int i = e / M, j = e % M;
      T v = i == j ? dg[i] : (i > j ? S[i * ld + j] : Num<T>::zero());
      Lout[(size_t)i * M + j] = Num<T>::st(v);
    }
  }
  if (logdet) {
    T l = Num<T>::zero();
    for (int i = tid; i < M; i += blockDim.x) l = add(l, log_tab(dg[i], tab));
    l = warp_sum(l);
    if (tx == 0) red[ty] = l;
    __syncthreads();
    if (ty == 0) {
      T s = tx < 32 ? red[tx] : Num<T>::zero();
      s = warp_sum(s);
      if (tx == 0) logdet[b] = (double)Num<T>::st(scale2(s, 1));
    }
  }
  if (!Ainv && !Xout) return;
  // in-place inverse of the lower factor, columns right to left:
  //   X_jj = 1/L_jj,  X_ij = -X_jj sum_{k=j+1..i} X_ik L_kj   (i > j)
  // column j's L entries are staged in tmp one step ahead, so each column costs two barriers.
  for (int k = M - 1 + tid; k < M; k += blockDim.x) tmp[k] = S[k * ld + (M - 1)];
  __syncthreads();
  for (int j = M - 1; j >= 0; --j) {
    // 8 threads per row, 128 rows per pass.  Row i reads only columns > j of S and the staged
    // column tmp, so writing X_ij into column j right away cannot race with other rows.
    for (int r0 = j + 1; r0 < M; r0 += 128) {
      int i = r0 + (tid >> 3), sl = tid & 7;
      T s = Num<T>::zero();
      if (i < M)
        for (int k = j + 1 + sl; k <= i; k += 8) s = fma_(S[i * ld + k], tmp[k], s);
#pragma unroll
      for (int m = 1; m < 8; m <<= 1) s = add(s, shfl_xor(s, m));
      if (i < M && sl == 0) S[i * ld + j] = neg(mul(di[j], s));
    }
    __syncthreads();
    if (tid == 0) S[j * ld + j] = di[j];
    if (j > 0)
      for (int k = j + tid; k < M; k += blockDim.x) tmp[k] = S[k * ld + (j - 1)];
    __syncthreads();
  }
  if (Xout) {
    // hand X = L^-1 (zeros above the diagonal) to the caller; the product X^T X is left to a
    // many-CTA GEMM instead of this single CTA
    Xout += (size_t)b * M * M;
    for (int e = tid; e < M * M; e += blockDim.x) {
      int i = e / M, j = e % M;
      Xout[e] = Num<T>::st(i >= j ? S[i * ld + j] : Num<T>::zero());
    }
    return;
  }
  // Ainv = X^T X  (X lower): Ainv_ij = sum_{k >= max(i,j)} X_ki X_kj
  Ainv += b * sI;
  for (int e = tid; e < M * (M + 1) / 2; e += blockDim.x) {
    int i = (int)((sqrtf(8.f * (float)e + 1.f) - 1.f) * 0.5f);
    if ((i + 1) * (i + 2) / 2 <= e) ++i;
    if (i * (i + 1) / 2 > e) --i;
    int j = e - i * (i + 1) / 2;   // j <= i
    T s = Num<T>::zero();
    for (int kk = i; kk < M; ++kk) s = fma_(S[kk * ld + i], S[kk * ld + j], s);
    typename Num<T>::store_t v = Num<T>::st(s);
    Ainv[(size_t)i * M + j] = v;
    Ainv[(size_t)j * M + i] = v;
  }
}

// gradient of tr(Mm Kzz), Kzz_ab = sf2 exp(-1/2 sum_q (z_aq - z_bq)^2 / l_q) (no jitter):
//   d/dlog sf2 = sum_ab Mm_ab K_ab;  d/dlog l_q = 1/2 sum_ab Mm_ab K_ab (z_aq-z_bq)^2 / l_q
//   d/dz_aq = sum_b (Mm_ab + Mm_ba) K_ab (z_bq - z_aq) / l_q
// (geepee/kernels.py:447-475).  Results are ADDED, scaled: g_sf += s_sf * ., g_ls += s_ls * ., g_z += .
// One CTA per pseudo-input a, a thread per b (b = threadIdx.x + k blockDim.x); the CTA sums its
// threads' d/dz_a in a fixed order and adds it into g_z[a] (one writer per element).  The sums
// over (a, b) of the log sf2 and log l terms leave each CTA as a partial (into
// part[a * (1 + Q)], fixed-order path) or by atomics.
constexpr int TK_MAXW = 8;   // warps per CTA
template <typename T, int QC>
__global__ void __launch_bounds__(TK_MAXW * 32) trace_kzz_kernel(int M, int Q, const typename Num<T>::store_t* Mm,
                                                                 const typename Num<T>::store_t* Z,
                                                                 const double* lls2, const double* lsf2, double s_sf,
                                                                 double s_ls, double* g_sf, double* g_ls, double* g_z,
                                                                 double* part) {
  typedef typename Num<T>::store_t S;
  extern __shared__ __align__(16) char smem_raw[];
  float2* tab = reinterpret_cast<float2*>(smem_raw);
  T* zs = reinterpret_cast<T*>(smem_raw + 256 * sizeof(float2));   // [M*Q]
  __shared__ T il[QC], lsf;
  __shared__ T red[TK_MAXW][1 + 2 * QC];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int a = blockIdx.x;
  // this thread's first M_ab and M_ba are loaded before the staging below
  S mab = S(0), mba = S(0);
  if (threadIdx.x < M) {
    mab = Mm[(size_t)a * M + threadIdx.x];
    mba = Mm[(size_t)threadIdx.x * M + a];
  }
  stage_async(reinterpret_cast<S*>(zs), Z, (long)M * Q, threadIdx.x, blockDim.x);
  load_exp_table(tab);
  __syncthreads();
  convert_in_place(zs, (long)M * Q, threadIdx.x, blockDim.x);
  if (threadIdx.x < Q) il[threadIdx.x] = exp_tab(neg(Num<T>::ld(static_cast<S>(lls2[threadIdx.x]))), tab);
  if (threadIdx.x == 31) lsf = Num<T>::ld(static_cast<S>(lsf2[0]));   // Q <= 8: thread 31 is free
  __syncthreads();
  T v[1 + 2 * QC];   // gs, gl[QC], gz[QC]
#pragma unroll
  for (int i = 0; i < 1 + 2 * QC; ++i) v[i] = Num<T>::zero();
  for (int b = threadIdx.x; b < M; b += blockDim.x) {
    if (b != (int)threadIdx.x) {
      mab = Mm[(size_t)a * M + b];
      mba = Mm[(size_t)b * M + a];
    }
    T r = Num<T>::zero();
    T d[QC];
#pragma unroll
    for (int q = 0; q < QC; ++q) {
      d[q] = q < Q ? sub(zs[b * Q + q], zs[a * Q + q]) : Num<T>::zero();   // z_b - z_a
      if (q < Q) r = fma_(mul(d[q], d[q]), il[q], r);
    }
    const T k = exp_tab(sub(lsf, scale2(r, -1)), tab);
    const T m1 = Num<T>::ld(mab);
    const T w = mul(m1, k);
    const T ws = mul(add(m1, Num<T>::ld(mba)), k);
    v[0] = add(v[0], w);
#pragma unroll
    for (int q = 0; q < QC; ++q) {
      if (q < Q) {
        const T dil = mul(d[q], il[q]);
        v[1 + q] = fma_(mul(w, d[q]), dil, v[1 + q]);
        v[1 + QC + q] = fma_(ws, dil, v[1 + QC + q]);
      }
    }
  }
  // the 1 + 2 QC warp sums in butterflies of eight (lane l then holds value c0 + l / 4), then
  // value i over the warps in order by thread i, which writes it
  constexpr int NV = 1 + 2 * QC;
#pragma unroll
  for (int c0 = 0; c0 < NV; c0 += 8) {
    T t[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) t[u] = c0 + u < NV ? v[(c0 + u) % NV] : Num<T>::zero();
    warp_sum_many<8>(t);
    if ((lane & 3) == 0 && c0 + (lane >> 2) < NV) red[warp][c0 + (lane >> 2)] = t[0];
  }
  __syncthreads();
  const int i = threadIdx.x;
  if (i < NV) {
    T t = red[0][i];
    for (int w = 1; w < nw; ++w) t = add(t, red[w][i]);
    if (i == 0) {
      const double vsf = s_sf * (double)Num<T>::st(t);
      if (part) part[(size_t)a * (1 + Q)] = vsf;
      else atomicAdd(g_sf, vsf);
    } else if (i <= QC) {
      const int q = i - 1;
      if (q < Q) {
        const double vl = s_ls * 0.5 * (double)Num<T>::st(t);
        if (part) part[(size_t)a * (1 + Q) + 1 + q] = vl;
        else atomicAdd(&g_ls[q], vl);
      }
    } else {
      const int q = i - 1 - QC;
      if (q < Q) g_z[a * Q + q] += (double)Num<T>::st(t);   // one writer per element (CTA a)
    }
  }
}

// Many tiny SPD matrices (n <= 8), one thread each: inverse and log-determinant by an
// in-register Cholesky.  The per-time-step Dy x Dy emission covariances of the GP
// state-space model (geepee/lik_layers.py:596-610 solve / slogdet / inv).
template <typename T>
__global__ void __launch_bounds__(128) small_spd_kernel(int B, int n, const typename Num<T>::store_t* A,
                                                        typename Num<T>::store_t* Ainv, double* logdet, int* info) {
  __shared__ float2 tab[256];
  load_exp_table(tab);
  __syncthreads();
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  const typename Num<T>::store_t* a = A + (size_t)b * n * n;
  T L[8][8];
  for (int i = 0; i < n; ++i)
    for (int j = 0; j <= i; ++j) L[i][j] = Num<T>::ld(a[i * n + j]);
  int bad = 0;
  T ld = Num<T>::zero();
  for (int k = 0; k < n && !bad; ++k) {
    T s = L[k][k];
    for (int j = 0; j < k; ++j) s = sub(s, mul(L[k][j], L[k][j]));
    if (!(Num<T>::approx(s) > 0.f)) { bad = k + 1; break; }
    T d = sqrt_(s);
    L[k][k] = d;
    ld = add(ld, log_tab(d, tab));
    T inv = recip(d);
    for (int i = k + 1; i < n; ++i) {
      T t = L[i][k];
      for (int j = 0; j < k; ++j) t = sub(t, mul(L[i][j], L[k][j]));
      L[i][k] = mul(t, inv);
    }
  }
  if (info) info[b] = bad;
  if (bad) return;
  if (logdet) logdet[b] = (double)Num<T>::st(scale2(ld, 1));
  if (!Ainv) return;
  // X = L^-1 (lower), then Ainv = X^T X
  T X[8][8];
  for (int j = 0; j < n; ++j) {
    X[j][j] = recip(L[j][j]);
    for (int i = j + 1; i < n; ++i) {
      T t = Num<T>::zero();
      for (int k = j; k < i; ++k) t = fma_(L[i][k], X[k][j], t);
      X[i][j] = neg(mul(t, recip(L[i][i])));
    }
  }
  typename Num<T>::store_t* o = Ainv + (size_t)b * n * n;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j <= i; ++j) {
      T t = Num<T>::zero();
      for (int k = i; k < n; ++k) t = fma_(X[k][i], X[k][j], t);
      typename Num<T>::store_t v = Num<T>::st(t);
      o[i * n + j] = v;
      o[j * n + i] = v;
    }
}

// Tile edge for a set of products with t8 8-wide / t16 16-wide tiles: 8 (256-thread CTAs,
// about four resident per SM) while the tiles fill at most two such waves, then 16 (one
// 1024-thread CTA per SM) up to two waves, then 32.  Small products are latency-bound: more,
// smaller CTAs start together and finish sooner (16-wide tiles of 2 x 2 outputs a thread, which
// convert each operand element half as often, measured slower: 9.6 against 6.2 us for one
// M = 100 product, and no faster for a group of six).
inline int gemm_tile_edge(long t8, long t16) {
  const long sms = gpk::sm_count();
  if (t8 <= 8 * sms) return 8;
  if (t16 <= 2 * sms) return 16;
  return 32;
}

template <typename T, int TBM, int KS, bool P2>
void gemm_go(int batch, int m, int n, int k, int tA, int tB, double alpha, const void* A, int lda, long sA,
             const void* B, int ldb, long sB, double beta, const void* E, int lde, long sE, void* C, int ldc, long sC,
             cudaStream_t st) {
  typedef typename Num<T>::store_t S;
  dim3 grid(gpk::ceil_div(n, TBM), gpk::ceil_div(m, TBM), batch);
  const size_t sm = 2 * KC * TBM * sizeof(T);
  auto kfn = gemm_kernel<T, TBM, KS, P2>;
  cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  kfn<<<grid, GemmShape<TBM>::NG * KS, sm, st>>>(m, n, k, tA, tB, alpha, (const S*)A, lda, sA, (const S*)B, ldb, sB,
                                                 beta, (const S*)E, lde, sE, (S*)C, ldc, sC);
}

// Tile choice: 32x32 tiles when they already fill the GPU twice over, 16x16 when those fill
// it once, else 8x8 tiles so that a small product still spreads over most SMs.  P2: A and B
// hold raw double-float pairs (8 bytes per element) instead of float64.
template <typename T, bool P2 = false>
int gemm_launch(int batch, int m, int n, int k, int tA, int tB, double alpha, const void* A, int lda, long sA,
                const void* B, int ldb, long sB, double beta, const void* E, int lde, long sE, void* C, int ldc,
                long sC, cudaStream_t st) {
  const int tbm = gemm_tile_edge((long)gpk::ceil_div(n, 8) * gpk::ceil_div(m, 8) * batch,
                                 (long)gpk::ceil_div(n, 16) * gpk::ceil_div(m, 16) * batch);
  if (tbm == 32)
    gemm_go<T, 32, 2, P2>(batch, m, n, k, tA, tB, alpha, A, lda, sA, B, ldb, sB, beta, E, lde, sE, C, ldc, sC, st);
  else if (tbm == 16)
    gemm_go<T, 16, 4, P2>(batch, m, n, k, tA, tB, alpha, A, lda, sA, B, ldb, sB, beta, E, lde, sE, C, ldc, sC, st);
  else
    gemm_go<T, 8, 4, P2>(batch, m, n, k, tA, tB, alpha, A, lda, sA, B, ldb, sB, beta, E, lde, sE, C, ldc, sC, st);
  return gpk::check_launch("gemm");
}

template <typename T, int TBM, int KS>
int gemm_group_go(const GemmGroupArgs& g, LincombGroupArgs& l, cudaStream_t st) {
  const size_t sm = 2 * KC * TBM * sizeof(T);
  const int nth = GemmShape<TBM>::NG * KS;
  // CTAs per linear combination: about two elements per thread, at most two waves
  l.first[0] = 0;
  for (int q = 0; q < l.count; ++q) {
    const gpk_lincomb_t& d = l.d[q];
    const long n = (long)d.rows * d.cols * (d.sum_batch ? 1 : d.batch);
    const long c = std::min<long>(std::max<long>((n + 2L * nth - 1) / (2L * nth), 1), 2L * gpk::sm_count());
    l.first[q + 1] = l.first[q] + (int)c;
  }
  const int grid = g.first[g.count] + l.first[l.count];
  if (grid == 0) return GPK_OK;
  auto kfn = gemm_group_kernel<T, TBM, KS>;
  cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  kfn<<<grid, nth, sm, st>>>(g, l);
  return gpk::check_launch("gemm_group");
}

template <typename T>
int gemm_group_launch(int count, const gpk_gemm_t* pr, int nlc, const gpk_lincomb_t* lcs, cudaStream_t st) {
  // the tile size is chosen for the whole group, as gemm_launch chooses it for one product
  long t8 = 0, t16 = 0;
  for (int p = 0; p < count; ++p) {
    t8 += (long)gpk::ceil_div(pr[p].n, 8) * gpk::ceil_div(pr[p].m, 8) * pr[p].batch;
    t16 += (long)gpk::ceil_div(pr[p].n, 16) * gpk::ceil_div(pr[p].m, 16) * pr[p].batch;
  }
  const int tbm = gemm_tile_edge(t8, t16);
  GemmGroupArgs g{};
  g.count = count;
  g.first[0] = 0;
  for (int p = 0; p < count; ++p) {
    g.pr[p] = pr[p];
    g.tiles_n[p] = gpk::ceil_div(pr[p].n, tbm);
    g.tiles_m[p] = gpk::ceil_div(pr[p].m, tbm);
    const long tiles = (long)g.tiles_n[p] * g.tiles_m[p] * pr[p].batch;
    if (g.first[p] + tiles > 0x7fffffffL) return gpk::fail(GPK_EUNSUPPORTED, "gemm_group: too many tiles");
    g.first[p + 1] = g.first[p] + (int)tiles;
  }
  LincombGroupArgs l{};
  l.count = nlc;
  for (int q = 0; q < nlc; ++q) l.d[q] = lcs[q];
  if (tbm == 32) return gemm_group_go<T, 32, 2>(g, l, st);
  if (tbm == 16) return gemm_group_go<T, 16, 4>(g, l, st);
  return gemm_group_go<T, 8, 4>(g, l, st);
}

}  // namespace

extern "C" int gpk_gemm(int prec, int batch, int m, int n, int k, int transA, int transB, double alpha,
                        const void* A, int lda, long strideA, const void* B, int ldb, long strideB, double beta,
                        void* C, int ldc, long strideC, void* stream) {
  GPK_NVTX("gpk_gemm");
  GPK_REQUIRE(batch >= 0 && m >= 0 && n >= 0 && k >= 0, "gemm: negative size");
  GPK_REQUIRE(batch <= 65535, "gemm: batch %d > 65535", batch);
  GPK_REQUIRE(C && (k == 0 || (A && B)), "gemm: null pointer");
  GPK_REQUIRE(lda >= (transA ? m : k) && ldb >= (transB ? k : n) && ldc >= n, "gemm: bad leading dimension");
  if (batch == 0 || m == 0 || n == 0) return GPK_OK;
  cudaStream_t st = gpk::as_stream(stream);
  if (prec == GPK_DF64)
    return gemm_launch<df64>(batch, m, n, k, transA, transB, alpha, A, lda, strideA, B, ldb, strideB, beta, C, ldc,
                             strideC, C, ldc, strideC, st);
  if (prec == GPK_FP32)
    return gemm_launch<float>(batch, m, n, k, transA, transB, alpha, A, lda, strideA, B, ldb, strideB, beta, C, ldc,
                              strideC, C, ldc, strideC, st);
  return gpk::fail(GPK_EINVAL, "gemm: unknown precision %d", prec);
}

extern "C" int gpk_gemm_ex(int prec, int batch, int m, int n, int k, int transA, int transB, double alpha,
                           const void* A, int lda, long strideA, const void* B, int ldb, long strideB, double beta,
                           const void* E, int lde, long strideE, void* C, int ldc, long strideC, void* stream) {
  GPK_NVTX("gpk_gemm_ex");
  GPK_REQUIRE(batch >= 0 && m >= 0 && n >= 0 && k >= 0, "gemm_ex: negative size");
  GPK_REQUIRE(batch <= 65535, "gemm_ex: batch %d > 65535", batch);
  GPK_REQUIRE(C && (k == 0 || (A && B)) && (beta == 0.0 || E), "gemm_ex: null pointer");
  GPK_REQUIRE(lda >= (transA ? m : k) && ldb >= (transB ? k : n) && ldc >= n && (beta == 0.0 || lde >= n),
              "gemm_ex: bad leading dimension");
  if (batch == 0 || m == 0 || n == 0) return GPK_OK;
  cudaStream_t st = gpk::as_stream(stream);
  if (prec == GPK_DF64)
    return gemm_launch<df64>(batch, m, n, k, transA, transB, alpha, A, lda, strideA, B, ldb, strideB, beta, E, lde,
                             strideE, C, ldc, strideC, st);
  if (prec == GPK_FP32)
    return gemm_launch<float>(batch, m, n, k, transA, transB, alpha, A, lda, strideA, B, ldb, strideB, beta, E, lde,
                              strideE, C, ldc, strideC, st);
  return gpk::fail(GPK_EINVAL, "gemm_ex: unknown precision %d", prec);
}

static int gemm_group_check(int count, const gpk_gemm_t* problems) {
  GPK_REQUIRE(count >= 0 && count <= GPK_GEMM_GROUP, "gemm_group: count %d outside [0,%d]", count, GPK_GEMM_GROUP);
  GPK_REQUIRE(count == 0 || problems, "gemm_group: null problem list");
  for (int p = 0; p < count; ++p) {
    const gpk_gemm_t& q = problems[p];
    GPK_REQUIRE(q.batch >= 0 && q.m >= 0 && q.n >= 0 && q.k >= 0 && q.batch <= 65535, "gemm_group[%d]: bad size", p);
    GPK_REQUIRE(q.C && (q.k == 0 || (q.A && q.B)) && (q.beta == 0.0 || q.E), "gemm_group[%d]: null pointer", p);
    GPK_REQUIRE(q.lda >= (q.transA ? q.m : q.k) && q.ldb >= (q.transB ? q.k : q.n) && q.ldc >= q.n &&
                    (q.beta == 0.0 || q.lde >= q.n),
                "gemm_group[%d]: bad leading dimension", p);
    GPK_REQUIRE(!q.sel || ((q.A2 || q.B2) && q.selbit >= 0 && q.selbit < 31),
                "gemm_group[%d]: a selector needs A2 or B2 and a bit in [0,30]", p);
    GPK_REQUIRE(!q.u == !q.v, "gemm_group[%d]: a rank-one addend needs both u and v", p);
  }
  return GPK_OK;
}

extern "C" int gpk_gemm_group(int prec, int count, const gpk_gemm_t* problems, void* stream) {
  GPK_NVTX("gpk_gemm_group");
  return gpk_level(prec, count, problems, 0, nullptr, stream);
}

extern "C" int gpk_level(int prec, int ngemm, const gpk_gemm_t* gemms, int nlc, const gpk_lincomb_t* lcs,
                         void* stream) {
  GPK_NVTX("gpk_level");
  if (const int rc = gemm_group_check(ngemm, gemms)) return rc;
  GPK_REQUIRE(nlc >= 0 && nlc <= GPK_LC_GROUP && (nlc == 0 || lcs), "level: %d linear combinations (max %d)", nlc,
              GPK_LC_GROUP);
  for (int q = 0; q < nlc; ++q) {
    long n = 0;
    if (const int rc = lincomb_check(&lcs[q], &n)) return rc;
  }
  if (ngemm == 0 && nlc == 0) return GPK_OK;
  cudaStream_t st = gpk::as_stream(stream);
  if (prec == GPK_DF64) return gemm_group_launch<df64>(ngemm, gemms, nlc, lcs, st);
  if (prec == GPK_FP32) return gemm_group_launch<float>(ngemm, gemms, nlc, lcs, st);
  return gpk::fail(GPK_EINVAL, "level: unknown precision %d", prec);
}

template <typename T, int RS, int CS, int NW>
int spd_factor_launch(int batch, int M, const void* A, T* Lw, double* logdet, int* info, cudaStream_t st) {
  typedef typename Num<T>::store_t S;
  const size_t sm = 256 * sizeof(float2) + ((size_t)((M + 1) >> 1) * (M + 32) * 2 + M + NW) * sizeof(T);
  auto k = spd_factor_kernel<T, RS, CS, NW>;
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k<<<batch, NW * 32, sm, st>>>(M, (const S*)A, (long)M * M, Lw, logdet, info);
  return gpk::check_launch("spd_factor");
}

template <typename T, int RS>
int trinv_launch(int batch, int M, const T* Lw, T* Xt, const int* info, cudaStream_t st) {
  const size_t sm = (size_t)M * M * sizeof(T);
  auto k = trinv_kernel<T, RS>;
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k<<<dim3(gpk::ceil_div(M, TW), batch), TW * 32, sm, st>>>(M, Lw, Xt, info);
  return gpk::check_launch("trinv");
}

// M <= 128: A^-1 = L^-T L^-1 through the factor, the column-parallel L^-1 and one GEMM.
// work: 2*batch*M*M elements of T (L, then X^T).  info is required (it gates trinv).
template <typename T>
int spd_inv_small(int batch, int M, const void* A, void* Ainv, double* logdet, int* info, void* work,
                  cudaStream_t st) {
  T* Lw = reinterpret_cast<T*>(work);
  T* Xt = Lw + (size_t)batch * M * M;
  int rc;
  if (M <= 32) rc = spd_factor_launch<T, 1, 2, 16>(batch, M, A, Lw, logdet, info, st);
  else if (M <= 64) rc = spd_factor_launch<T, 2, 4, 16>(batch, M, A, Lw, logdet, info, st);
  else if (M <= 96) rc = spd_factor_launch<T, 3, 6, 16>(batch, M, A, Lw, logdet, info, st);
  else if (M <= 112) rc = spd_factor_launch<T, 4, 7, 16>(batch, M, A, Lw, logdet, info, st);
  else rc = spd_factor_launch<T, 4, 8, 16>(batch, M, A, Lw, logdet, info, st);
  if (rc) return rc;
  if (M <= 32) rc = trinv_launch<T, 1>(batch, M, Lw, Xt, info, st);
  else if (M <= 64) rc = trinv_launch<T, 2>(batch, M, Lw, Xt, info, st);
  else if (M <= 96) rc = trinv_launch<T, 3>(batch, M, Lw, Xt, info, st);
  else rc = trinv_launch<T, 4>(batch, M, Lw, Xt, info, st);
  if (rc) return rc;
  const long s = (long)M * M;
  // A^-1 = X^T X = Xt Xt^T
  return gemm_launch<T, true>(batch, M, M, M, 0, 1, 1.0, Xt, M, s, Xt, M, s, 0.0, nullptr, M, 0, Ainv, M, s, st);
}

template <typename T, bool GMEM>
int chol_launch(int batch, int M, const void* A, void* Ainv, void* L, double* logdet, int* info, void* work,
                void* Xout, cudaStream_t st) {
  typedef typename Num<T>::store_t S;
  long s = (long)M * M;
  size_t sm = 256 * 8 + ((GMEM ? 0 : (size_t)M * (M + 1)) + 3 * M + 32) * sizeof(T);
  auto k = chol_inv_kernel<T, GMEM>;
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k<<<batch, 1024, sm, st>>>(M, (const S*)A, s, (S*)Ainv, s, (S*)L, s, logdet, info, (S*)work, (S*)Xout);
  return gpk::check_launch("chol_inv");
}

extern "C" int gpk_chol_inv_ws(int prec, int batch, int M, const void* A, void* Ainv, void* L, double* logdet,
                               int* info, void* work, void* stream) {
  GPK_NVTX("gpk_chol_inv_ws");
  GPK_REQUIRE(batch >= 0 && batch <= 65535 && M >= 1 && M <= 4096, "chol_inv: M=%d outside [1,4096]", M);
  GPK_REQUIRE(A, "chol_inv: null input");
  GPK_REQUIRE(M <= 128 || work, "chol_inv: M=%d > 128 needs a workspace of batch*M*M elements", M);
  if (batch == 0) return GPK_OK;
  cudaStream_t st = gpk::as_stream(stream);
  const bool gm = M > 128;
  if (prec == GPK_DF64)
    return gm ? chol_launch<df64, true>(batch, M, A, Ainv, L, logdet, info, work, nullptr, st)
              : chol_launch<df64, false>(batch, M, A, Ainv, L, logdet, info, work, nullptr, st);
  if (prec == GPK_FP32)
    return gm ? chol_launch<float, true>(batch, M, A, Ainv, L, logdet, info, work, nullptr, st)
              : chol_launch<float, false>(batch, M, A, Ainv, L, logdet, info, work, nullptr, st);
  return gpk::fail(GPK_EINVAL, "chol_inv: unknown precision %d", prec);
}

extern "C" int gpk_chol_inv(int prec, int batch, int M, const void* A, void* Ainv, void* L, double* logdet, int* info,
                            void* stream) {
  GPK_NVTX("gpk_chol_inv");
  GPK_REQUIRE(M <= 128, "chol_inv: M=%d > 128 needs gpk_chol_inv_ws", M);
  return gpk_chol_inv_ws(prec, batch, M, A, Ainv, L, logdet, info, nullptr, stream);
}

extern "C" int gpk_spd_inv(int prec, int batch, int M, const void* A, void* Ainv, double* logdet, int* info,
                           void* work, void* stream) {
  GPK_NVTX("gpk_spd_inv");
  GPK_REQUIRE(batch >= 0 && batch <= 65535 && M >= 1 && M <= 4096, "spd_inv: M=%d outside [1,4096]", M);
  GPK_REQUIRE(A && Ainv && info && work, "spd_inv: null pointer");
  if (batch == 0) return GPK_OK;
  cudaStream_t st = gpk::as_stream(stream);
  if (prec != GPK_DF64 && prec != GPK_FP32) return gpk::fail(GPK_EINVAL, "spd_inv: unknown precision %d", prec);
  if (M > 128)
    return prec == GPK_DF64
               ? chol_launch<df64, true>(batch, M, A, Ainv, nullptr, logdet, info, work, nullptr, st)
               : chol_launch<float, true>(batch, M, A, Ainv, nullptr, logdet, info, work, nullptr, st);
  return prec == GPK_DF64 ? spd_inv_small<df64>(batch, M, A, Ainv, logdet, info, work, st)
                          : spd_inv_small<float>(batch, M, A, Ainv, logdet, info, work, st);
}

// ---- gpk_spd_inv_static: gpk_spd_inv with its workspace in a file-scope device array ----
// Limit: M <= 128, batch <= 65535 and batch * M * M <= SPD_STATIC_ELEMS (e.g. 8 matrices of
// 128 x 128).  Nothing in the array needs to start at zero (every element a call reads was
// written earlier in the same call).  There is one array per device: calls that overlap on the
// device (different streams or host threads) race on it.
constexpr long SPD_STATIC_ELEMS = 8L * 128 * 128;
static_assert(sizeof(df64) <= 8 && sizeof(float) <= 8, "the array holds 2 SPD_STATIC_ELEMS elements of <= 8 bytes");
static __device__ __align__(256) unsigned char g_spd_scratch[2 * SPD_STATIC_ELEMS * 8];

namespace {
// Device address of g_spd_scratch on the current device, looked up on every call: the lookup
// is cheap once the module is loaded, and a cached address would go stale when the device's
// context is torn down and created again (cudaDeviceReset), which reloads the module.
int spd_scratch(void** out) {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_spd_scratch);
  if (e != cudaSuccess || !p)
    return gpk::fail(GPK_ECUDA, "spd_inv_static: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
  *out = p;
  return GPK_OK;
}
}  // namespace

extern "C" int gpk_spd_inv_static(int prec, int batch, int M, const void* A, void* Ainv, double* logdet, int* info,
                                  void* stream) {
  GPK_NVTX("gpk_spd_inv_static");
  GPK_REQUIRE(batch >= 0 && batch <= 65535 && M >= 1 && M <= 128,
              "spd_inv_static: batch=%d outside [0,65535] or M=%d outside [1,128]", batch, M);
  GPK_REQUIRE((long)batch * M * M <= SPD_STATIC_ELEMS, "spd_inv_static: batch*M*M = %ld > %ld",
              (long)batch * M * M, SPD_STATIC_ELEMS);
  GPK_REQUIRE(A && Ainv && info, "spd_inv_static: null pointer");
  if (prec != GPK_DF64 && prec != GPK_FP32) return gpk::fail(GPK_EINVAL, "spd_inv_static: unknown precision %d", prec);
  if (batch == 0) return GPK_OK;
  void* work = nullptr;
  const int rc = spd_scratch(&work);
  if (rc) return rc;
  cudaStream_t st = gpk::as_stream(stream);
  return prec == GPK_DF64 ? spd_inv_small<df64>(batch, M, A, Ainv, logdet, info, work, st)
                          : spd_inv_small<float>(batch, M, A, Ainv, logdet, info, work, st);
}

template <typename T, int QC>
int trace_launch(int M, int Q, const void* Mm, const void* Z, const double* lls2, const double* lsf2, double s_sf,
                 double s_ls, double* g_sf, double* g_ls, double* g_z, double* work, cudaStream_t st) {
  typedef typename Num<T>::store_t S;
  const size_t sm = 256 * sizeof(float2) + (size_t)M * Q * sizeof(T);
  auto k = trace_kzz_kernel<T, QC>;
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k<<<M, 32 * std::min(TK_MAXW, gpk::ceil_div(M, 32)), sm, st>>>(M, Q, (const S*)Mm, (const S*)Z, lls2, lsf2, s_sf, s_ls, g_sf, g_ls,
                                             g_z, work);
  int rc = gpk::check_launch("trace_kzz");
  if (rc != GPK_OK || !work) return rc;
  gpk::RedPlan plan{};
  plan.add(g_sf, 1);
  plan.add(g_ls, Q);
  return gpk::reduce_partials(work, M, plan, st);
}

long trace_kzz_work_elems(int M, int Q) { return (long)M * (1 + Q); }

extern "C" int gpk_trace_kzz(int prec, int M, int Q, const void* Mm, const void* Z, const double* lls2,
                             const double* lsf2, double s_sf, double s_ls, double* g_sf, double* g_ls, double* g_z,
                             void* stream) {
  GPK_NVTX("gpk_trace_kzz");
  return gpk_trace_kzz_ws(prec, M, Q, Mm, Z, lls2, lsf2, s_sf, s_ls, g_sf, g_ls, g_z, nullptr, 0, stream);
}

extern "C" int gpk_trace_kzz_ws(int prec, int M, int Q, const void* Mm, const void* Z, const double* lls2,
                                const double* lsf2, double s_sf, double s_ls, double* g_sf, double* g_ls, double* g_z,
                                double* work, long work_elems, void* stream) {
  GPK_NVTX("gpk_trace_kzz_ws");
  GPK_REQUIRE(M >= 1 && Q >= 1 && Q <= 8, "trace_kzz: bad sizes M=%d Q=%d", M, Q);
  GPK_REQUIRE((size_t)M * Q * 8 <= 200 * 1024, "trace_kzz: M*Q=%d too large", M * Q);
  GPK_REQUIRE(Mm && Z && lls2 && lsf2 && g_sf && g_ls && g_z, "trace_kzz: null pointer");
  GPK_REQUIRE(!work || work_elems >= trace_kzz_work_elems(M, Q), "trace_kzz: workspace of %ld doubles, %ld needed",
              work_elems, trace_kzz_work_elems(M, Q));
  cudaStream_t st = gpk::as_stream(stream);
  if (prec == GPK_DF64)
    return Q <= 2 ? trace_launch<df64, 2>(M, Q, Mm, Z, lls2, lsf2, s_sf, s_ls, g_sf, g_ls, g_z, work, st)
                  : trace_launch<df64, 8>(M, Q, Mm, Z, lls2, lsf2, s_sf, s_ls, g_sf, g_ls, g_z, work, st);
  if (prec == GPK_FP32)
    return Q <= 2 ? trace_launch<float, 2>(M, Q, Mm, Z, lls2, lsf2, s_sf, s_ls, g_sf, g_ls, g_z, work, st)
                  : trace_launch<float, 8>(M, Q, Mm, Z, lls2, lsf2, s_sf, s_ls, g_sf, g_ls, g_z, work, st);
  return gpk::fail(GPK_EINVAL, "trace_kzz: unknown precision %d", prec);
}

extern "C" int gpk_small_spd(int prec, int batch, int n, const void* A, void* Ainv, double* logdet, int* info,
                             void* stream) {
  GPK_NVTX("gpk_small_spd");
  GPK_REQUIRE(batch >= 0 && n >= 1 && n <= 8, "small_spd: n=%d outside [1,8]", n);
  GPK_REQUIRE(A, "small_spd: null input");
  if (batch == 0) return GPK_OK;
  cudaStream_t st = gpk::as_stream(stream);
  int grid = gpk::ceil_div(batch, 128);
  if (prec == GPK_DF64)
    small_spd_kernel<df64><<<grid, 128, 0, st>>>(batch, n, (const double*)A, (double*)Ainv, logdet, info);
  else if (prec == GPK_FP32)
    small_spd_kernel<float><<<grid, 128, 0, st>>>(batch, n, (const float*)A, (float*)Ainv, logdet, info);
  else
    return gpk::fail(GPK_EINVAL, "small_spd: unknown precision %d", prec);
  return gpk::check_launch("small_spd");
}

// the translation unit's bounds word (debug build; 0 otherwise)
GPK_BOUNDS_READER(dense)
