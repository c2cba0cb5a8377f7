// ARD exponentiated-quadratic kernel matrices and the deterministic-input sparse-GP
// layer (first DGP layer / SGPR): fused forward contractions and the per-row backward.
#include "common.cuh"

namespace {

constexpr int DMAXK = 64;   // max input dimension
constexpr int DO_MAX = 4;   // max output dimension of a layer

template <typename T>
struct Hyp {
  T inv_l2[DMAXK];   // 1/ell^2
  T lsf;             // log sf^2
  T sf2;
};

template <typename T>
__device__ void load_hyp(Hyp<T>& h, const double* lls2, const double* lsf2, int D, const float2* tab) {
  typedef typename Num<T>::store_t S;
  for (int d = threadIdx.x; d < D; d += blockDim.x)
    h.inv_l2[d] = exp_tab(neg(Num<T>::ld(static_cast<S>(lls2[d]))), tab);
  if (threadIdx.x == 0) {
    h.lsf = Num<T>::ld(static_cast<S>(lsf2[0]));
    h.sf2 = exp_tab(h.lsf, tab);
  }
}

// K[n,m] = exp(lsf - 1/2 sum_d (x-z)^2 / l_d) (+ jitter on the diagonal).  A CTA takes KR rows
// and KC columns: those rows of x and columns' Z arrive in shared memory by asynchronous copies
// and are converted once (not once per element), then 256 threads sweep the KR x KC block.
constexpr int KR = 8, KC = 128;
template <typename T>
__global__ void __launch_bounds__(256) kern_matrix_kernel(int N, int M, int D, const typename Num<T>::store_t* x,
                                                          int ldx, const typename Num<T>::store_t* z, int ldz,
                                                          const double* lls2, const double* lsf2, double jitter,
                                                          typename Num<T>::store_t* K, int ldk) {
  typedef typename Num<T>::store_t S;
  extern __shared__ __align__(16) char smem_raw[];
  float2* tab = reinterpret_cast<float2*>(smem_raw);
  Hyp<T>* h = reinterpret_cast<Hyp<T>*>(smem_raw + 256 * sizeof(float2));
  T* xs = reinterpret_cast<T*>(smem_raw + 256 * sizeof(float2) + sizeof(Hyp<T>));   // [KR][D]
  T* zs = xs + KR * D;                                                                  // [KC][D]
  const int tid = threadIdx.x;
  const int m0 = blockIdx.x * KC, n0 = blockIdx.y * KR;
  const int nr = min(KR, N - n0), nc = min(KC, M - m0);
  for (int e = tid; e < nr * D; e += 256) {
    const int r = e / D, d = e - r * D;
    const unsigned dst = (unsigned)__cvta_generic_to_shared(reinterpret_cast<S*>(xs) + e);
    const S* src = x + (size_t)(n0 + r) * ldx + d;
    if (sizeof(S) == 8) asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(dst), "l"(src));
    else asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(dst), "l"(src));
  }
  for (int e = tid; e < nc * D; e += 256) {
    const int c = e / D, d = e - c * D;
    const unsigned dst = (unsigned)__cvta_generic_to_shared(reinterpret_cast<S*>(zs) + e);
    const S* src = z + (size_t)(m0 + c) * ldz + d;
    if (sizeof(S) == 8) asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(dst), "l"(src));
    else asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(dst), "l"(src));
  }
  asm volatile("cp.async.wait_all;\n" ::: "memory");
  load_exp_table(tab);
  __syncthreads();
  convert_in_place(xs, (long)nr * D, tid, 256);
  convert_in_place(zs, (long)nc * D, tid, 256);
  load_hyp(*h, lls2, lsf2, D, tab);
  __syncthreads();
  for (int e = tid; e < nr * nc; e += 256) {
    const int r = e / nc, c = e - r * nc;
    const int n = n0 + r, m = m0 + c;
    T rr = Num<T>::zero();
    for (int d = 0; d < D; ++d) {
      const T df = sub(xs[r * D + d], zs[c * D + d]);
      rr = fma_(mul(df, df), h->inv_l2[d], rr);
    }
    T k = exp_tab(sub(h->lsf, scale2(rr, -1)), tab);
    if (jitter != 0.0 && n == m) k = add(k, Num<T>::ld(static_cast<S>(jitter)));
    K[(size_t)n * ldk + m] = Num<T>::st(k);
  }
}

// Deterministic-input layer forward for rows n:
//   k_n = K(x_n, Z);  m_nd = k_n . A_d;  Bk_ndb = sum_a B_d[a,b] k_na;  v_nd = sf2 + k_n . Bk_nd
// (geepee/aep_models.py:142-158, base_models.py:265-284).
//
// A CTA takes tiles of FT rows for one output d (blockIdx.y).  The rows' kernel values go to
// shared memory; then, for each block of 128 columns b, every thread owns one column and FT/2
// rows of Bk and
// runs their sums over a from shared memory, while B_d streams through shared memory in
// chunks of FKA rows.  The next chunk's global loads are issued before the current chunk is
// used (register double buffer), so the stream costs one memory latency per tile, not one
// per chunk.  m and v are reduced over the columns by warp shuffles.
constexpr int FT = 8;      // rows per tile
constexpr int FKA = 32;    // rows of B_d per staged chunk
constexpr int FCB = 128;   // columns per block
constexpr int FNL = FKA * FCB / 256;   // staged elements per thread per chunk
template <typename T>
__global__ void __launch_bounds__(256) det_fwd_kernel(int N, int M, int D, int Dout,
                                                      const typename Num<T>::store_t* x, int ldx,
                                                      const typename Num<T>::store_t* z, const double* lls2,
                                                      const double* lsf2, const typename Num<T>::store_t* A,
                                                      const typename Num<T>::store_t* B,
                                                      typename Num<T>::store_t* kfu,
                                                      typename Num<T>::store_t* Bk,
                                                      typename Num<T>::store_t* m_out,
                                                      typename Num<T>::store_t* v_out, int zstage) {
  typedef typename Num<T>::store_t S;
  extern __shared__ __align__(16) char smem_raw[];
  float2* tab = reinterpret_cast<float2*>(smem_raw);
  Hyp<T>* h = reinterpret_cast<Hyp<T>*>(smem_raw + 256 * sizeof(float2));
  T* kr = reinterpret_cast<T*>(smem_raw + 256 * sizeof(float2) + sizeof(Hyp<T>));   // [FT][M]
  T* Bc = kr + FT * M;                       // [FKA][FCB]
  T* red = Bc + FKA * FCB;                   // [8 warps][DO_MAX][FT/2][2]
  T* xs = red + 8 * DO_MAX * FT;             // [FT][D]
  T* zs = xs + FT * D;                       // [M][D] when staged
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int col = tid & (FCB - 1), rh = tid >> 7;   // column in the block, row half
  load_exp_table(tab);
  if (zstage)
    for (int i = tid; i < M * D; i += 256) zs[i] = Num<T>::ld(z[i]);
  __syncthreads();
  load_hyp(*h, lls2, lsf2, D, tab);
  const int d = blockIdx.y;   // this CTA's output
  const int nca = (M + FKA - 1) / FKA, ncb = (M + FCB - 1) / FCB, nq = ncb * nca;
  const size_t MM = (size_t)M * M;
  auto issue = [&](int q, S* raw) {
    const int cb0 = (q / nca) * FCB, a0 = (q % nca) * FKA;
    const S* Bd = B + (size_t)d * MM;
#pragma unroll
    for (int u = 0; u < FNL; ++u) {
      const int e = tid + u * 256, aa = e / FCB, cc = e % FCB;
      const int a = a0 + aa, b = cb0 + cc;
      raw[u] = (a < M && b < M) ? Bd[(size_t)a * M + b] : S(0);
    }
  };
  for (int n0 = blockIdx.x * FT; n0 < N; n0 += gridDim.x * FT) {
    S raw[FNL];
    issue(0, raw);   // the first chunk's loads overlap the kernel values below
    for (int i = tid; i < FT * D; i += 256) {
      const int r = i / D, q = i - r * D, n = n0 + r;
      xs[i] = n < N ? Num<T>::ld(x[(size_t)n * ldx + q]) : Num<T>::zero();
    }
    __syncthreads();
    for (int i = tid; i < FT * M; i += 256) {
      const int r = i / M, mm = i - r * M, n = n0 + r;
      T k = Num<T>::zero();
      if (n < N) {
        T rr = Num<T>::zero();
        for (int q = 0; q < D; ++q) {
          const T zq = zstage ? zs[mm * D + q] : Num<T>::ld(z[(size_t)mm * D + q]);
          const T df = sub(xs[r * D + q], zq);
          rr = fma_(mul(df, df), h->inv_l2[q], rr);
        }
        k = exp_tab(sub(h->lsf, scale2(rr, -1)), tab);
        if (kfu && d == 0) kfu[(size_t)n * M + mm] = Num<T>::st(k);
      }
      kr[i] = k;
    }
    T acc[FT / 2], pm[FT / 2], pv[FT / 2];
    for (int q = 0; q < nq; ++q) {
      const int cbi = q / nca, ai = q % nca;
      const int a0 = ai * FKA, b = cbi * FCB + col;
      __syncthreads();   // the previous chunk is consumed (and kr is complete)
#pragma unroll
      for (int u = 0; u < FNL; ++u) Bc[tid + u * 256] = Num<T>::ld(raw[u]);
      __syncthreads();
      if (q + 1 < nq) issue(q + 1, raw);
      if (q == 0) {
#pragma unroll
        for (int r = 0; r < FT / 2; ++r) pm[r] = pv[r] = Num<T>::zero();
      }
      if (ai == 0) {
#pragma unroll
        for (int r = 0; r < FT / 2; ++r) acc[r] = Num<T>::zero();
      }
      const int ka = min(FKA, M - a0);
      const T* kt = kr + (rh * (FT / 2)) * M + a0;
#pragma unroll 4
      for (int aa = 0; aa < ka; ++aa) {
        const T bab = Bc[aa * FCB + col];
#pragma unroll
        for (int r = 0; r < FT / 2; ++r) acc[r] = fma_(bab, kt[r * M + aa], acc[r]);
      }
      if (ai == nca - 1 && b < M) {
        const T ad = Num<T>::ld(A[(size_t)d * M + b]);
#pragma unroll
        for (int r = 0; r < FT / 2; ++r) {
          const int rl = rh * (FT / 2) + r, n = n0 + rl;
          if (n < N && Bk) Bk[((size_t)n * Dout + d) * M + b] = Num<T>::st(acc[r]);
          const T kb = kr[rl * M + b];
          pm[r] = fma_(kb, ad, pm[r]);
          pv[r] = fma_(kb, acc[r], pv[r]);
        }
      }
      if (ai == nca - 1 && cbi == ncb - 1) {
#pragma unroll
        for (int r = 0; r < FT / 2; ++r) {
          const T sm = warp_sum(pm[r]), sv = warp_sum(pv[r]);
          if (lane == 0) {
            red[((warp * DO_MAX + d) * (FT / 2) + r) * 2] = sm;
            red[((warp * DO_MAX + d) * (FT / 2) + r) * 2 + 1] = sv;
          }
        }
      }
    }
    __syncthreads();
    for (int rl = tid; rl < FT; rl += 256) {
      const int n = n0 + rl;
      const int hh = rl / (FT / 2), r = rl - hh * (FT / 2);
      if (n < N) {
        T mm = Num<T>::zero(), vv = Num<T>::zero();
#pragma unroll
        for (int w = 0; w < 4; ++w) {   // the four warps of row half hh
          const int ww = hh * 4 + w;
          mm = add(mm, red[((ww * DO_MAX + d) * (FT / 2) + r) * 2]);
          vv = add(vv, red[((ww * DO_MAX + d) * (FT / 2) + r) * 2 + 1]);
        }
        if (m_out) m_out[(size_t)n * Dout + d] = Num<T>::st(mm);
        if (v_out) v_out[(size_t)n * Dout + d] = Num<T>::st(add(h->sf2, vv));
      }
    }
  }
}

// The deterministic-input layer's contractions from given kernel values kfu [N,M]:
//   m_nd = kfu_n . A_d;  Bk_ndb = sum_a B_d[a,b] kfu_na;  v_nd = sf2 + kfu_n . Bk_nd
// (geepee/aep_models.py:142-158 once Kfu is formed).  A CTA takes CR rows; warp w works on row
// w % CR and column half w / CR, lane l on columns b = 64 h + l + 32 j (j < 2), for all DB
// outputs, so each thread runs 2 DB independent sums over a.  All of B (Dout M^2) and the CTA's
// kernel rows sit in shared memory (asynchronous copies, converted in place, 8-byte aligned so
// that each element is one shared-memory access); m and v are warp sums, then the two halves'
// sums are added in a fixed order.
constexpr int CR = 8;              // rows per CTA
constexpr int CT = CR * 2 * 32;    // threads: (row, column half) per warp
template <typename T, int DB>
__global__ void __launch_bounds__(CT) det_contract_kernel(int N, int M, int Dout,
                                                          const typename Num<T>::store_t* kfu,
                                                          const double* lsf2,
                                                          const typename Num<T>::store_t* A,
                                                          const typename Num<T>::store_t* B,
                                                          typename Num<T>::store_t* Bk,
                                                          typename Num<T>::store_t* m_out,
                                                          typename Num<T>::store_t* v_out, int b_pairs) {
  typedef typename Num<T>::store_t S;
  extern __shared__ __align__(16) char smem_raw[];
  float2* tab = reinterpret_cast<float2*>(smem_raw);
  T* Bs = reinterpret_cast<T*>(smem_raw + 256 * sizeof(float2));   // [Dout][M][M]
  T* kr = Bs + (size_t)Dout * M * M;                                 // [CR][M]
  T* red = kr + (size_t)CR * M;                                      // [2][CR][DB][2] half sums
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const int r = w % CR, h = w / CR;
  const int n0 = blockIdx.x * CR, n = n0 + r;
  const int nB = Dout * M * M, nr = min(CR, N - n0);
  stage_async(reinterpret_cast<S*>(Bs), B, nB, tid, CT);
  stage_async(reinterpret_cast<S*>(kr), kfu + (size_t)n0 * M, (long)nr * M, tid, CT);
  load_exp_table(tab);
  __syncthreads();
  if (!b_pairs) convert_in_place(Bs, nB, tid, CT);   // pairs arrive in the compute type already
  convert_in_place(kr, (long)nr * M, tid, CT);
  __syncthreads();
  const bool live = n < N;   // warp-uniform; a dead row still reaches the barrier below
  const T* k = kr + (size_t)(live ? r : 0) * M;
  // columns past M read the row's last column (in bounds) and are never stored
  const int c0 = min(64 * h + lane, M - 1), c1 = min(64 * h + lane + 32, M - 1);
  T acc[DB][2];
#pragma unroll
  for (int d = 0; d < DB; ++d) acc[d][0] = acc[d][1] = Num<T>::zero();
  // output d's columns of B; outputs past Dout (DB = 4 for Dout = 3) read output 0's, in
  // bounds, and are never stored
  const T* B0[DB];
  const T* B1[DB];
#pragma unroll
  for (int d = 0; d < DB; ++d) {
    const size_t off = (size_t)(d < Dout ? d : 0) * M * M;
    B0[d] = Bs + off + c0;
    B1[d] = Bs + off + c1;
  }
  for (int a = 0; a < M; ++a) {
    const T ka = k[a];
    const size_t ra = (size_t)a * M;
#pragma unroll
    for (int d = 0; d < DB; ++d) {
      // det_fwd's operand order, so that the sums match its arithmetic
      acc[d][0] = fma_(ld_al8(B0[d] + ra), ka, acc[d][0]);
      acc[d][1] = fma_(ld_al8(B1[d] + ra), ka, acc[d][1]);
    }
  }
  T pm[DB], pv[DB];
#pragma unroll
  for (int d = 0; d < DB; ++d) {
    pm[d] = pv[d] = Num<T>::zero();
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const int b = 64 * h + lane + 32 * j;
      if (live && b < M && d < Dout) {
        if (Bk) Bk[((size_t)n * Dout + d) * M + b] = Num<T>::st(acc[d][j]);
        pm[d] = fma_(k[b], Num<T>::ld(A[(size_t)d * M + b]), pm[d]);
        pv[d] = fma_(k[b], acc[d][j], pv[d]);
      }
    }
    pm[d] = warp_sum(pm[d]);
    pv[d] = warp_sum(pv[d]);
    if (lane == 0) {
      red[((h * CR + r) * DB + d) * 2] = pm[d];
      red[((h * CR + r) * DB + d) * 2 + 1] = pv[d];
    }
  }
  __syncthreads();
  if (h == 0 && lane == 0 && live) {
    const T sf2 = exp_tab(Num<T>::ld(static_cast<S>(lsf2[0])), tab);
#pragma unroll
    for (int d = 0; d < DB; ++d) {
      if (d < Dout) {
        const T mm = add(red[((0 * CR + r) * DB + d) * 2], red[((1 * CR + r) * DB + d) * 2]);
        const T vv = add(red[((0 * CR + r) * DB + d) * 2 + 1], red[((1 * CR + r) * DB + d) * 2 + 1]);
        if (m_out) m_out[(size_t)n * Dout + d] = Num<T>::st(mm);
        if (v_out) v_out[(size_t)n * Dout + d] = Num<T>::st(add(sf2, vv));
      }
    }
  }
}

size_t det_contract_smem(int M, int Dout, size_t tsz) {
  return 256 * sizeof(float2) + ((size_t)Dout * M * M + (size_t)CR * M + 2 * CR * DO_MAX * 2) * tsz;
}

// elements of one det_bwd row buffer: RG rows of kfu (or dkfu) and Bk, x, dm, dv
__host__ __device__ inline int det_bwd_rowbuf(int RG, int M, int D, int Dk) { return RG * (M * (1 + Dk) + D + 2 * Dk); }

// Deterministic-input layer backward, per row (geepee/aep_models.py:451-460 with
// kfucompDer, kernels.py:381-399):
//   dkfu_nb = sum_d dm_nd A_db + 2 sum_d dv_nd Bk_ndb,   L_nb = dkfu_nb kfu_nb
//   dsf2 += sum L / sf2;  dl_q += sum L (x-z)^2 / l^{3/2};  dZ_bq += sum_n L (x_nq - z_bq)/l_q
//   dA_db += sum_n dm_nd kfu_nb;   dx_nq = -sum_b L_nb (x_nq - z_bq)/l_q   (optional)
// Threads are (b, row group): threadIdx.x is the pseudo-input b, threadIdx.y one of RG row
// groups; a CTA takes a contiguous range of rows, RG at a time, whose kfu, Bk, x, dm, dv rows
// are copied into shared memory (double-buffered: the next RG rows' copies are in flight while
// these compute) and converted once; Z and A likewise at the start.  Per-b sums (dZ, dA) are
// reduced over the row groups in shared memory and flushed with one write (or atomic) per CTA;
// dsf2 and dl by one CTA reduction.
// DB outputs (Dout <= DB, every one of the first DB live unless DB = DO_MAX) and EX (D == DC)
// are compile-time, so that the per-row loops carry no branch between independent sums.
template <typename T, int DC, int DB, bool EX>
__global__ void __launch_bounds__(512) det_bwd_kernel(int N, int M, int D, int Dout,
                                                      const typename Num<T>::store_t* x, int ldx,
                                                      const typename Num<T>::store_t* z, const double* lls2,
                                                      const double* lsf2, const typename Num<T>::store_t* A,
                                                      const typename Num<T>::store_t* kfu,
                                                      const typename Num<T>::store_t* Bk,
                                                      const typename Num<T>::store_t* dm,
                                                      const typename Num<T>::store_t* dv,
                                                      const typename Num<T>::store_t* dkfu, double* dsf2,
                                                      double* dl, double* dZ, double* dA,
                                                      typename Num<T>::store_t* dx, double* part,
                                                      long part_stride) {
  typedef typename Num<T>::store_t S;
  extern __shared__ __align__(16) char smem_raw[];
  float2* tab = reinterpret_cast<float2*>(smem_raw);
  Hyp<T>* h = reinterpret_cast<Hyp<T>*>(smem_raw + 256 * sizeof(float2));
  const int RG = blockDim.y, XW = blockDim.x >> 5;
  const int Dk = dkfu ? 0 : Dout;   // outputs whose A, Bk, dm, dv are read
  const int BS = det_bwd_rowbuf(RG, M, D, Dk);
  T* zs = reinterpret_cast<T*>(smem_raw + 256 * sizeof(float2) + sizeof(Hyp<T>));   // [M][D]
  T* as = zs + (size_t)M * D;                // [Dk][M]
  T* buf = as + (size_t)Dk * M;              // [2][BS]: RG rows of kfu (or dkfu), Bk, x, dm, dv
  T* red = buf + 2 * (size_t)BS;             // [RG][XW][DC] (dx) / [RG][blockDim.x][DC+DO_MAX]
  const int b = threadIdx.x, rg = threadIdx.y, lane = threadIdx.x & 31, xw = threadIdx.x >> 5;
  const int tid = rg * blockDim.x + b, nth = blockDim.x * blockDim.y;
  const int nbeg = (int)((long)N * blockIdx.x / gridDim.x), nend = (int)((long)N * (blockIdx.x + 1) / gridDim.x);
  // The rows of a pass arrive by asynchronous copies into one of two buffers while the other
  // pass computes; each thread converts the elements it copied (one conversion site for all
  // of them), and a barrier publishes them.  Buffer layout (nr <= RG rows from n0):
  //   [0, RG M) kfu or dkfu rows | [RG M, RG M (1+Dk)) Bk rows | RG D x rows | RG Dk dm | RG Dk dv
  auto rowbuf = [&](int i, int n0, int nr, bool convert) {
    T* B0 = buf + (size_t)(i & 1) * BS;
    S* R0 = reinterpret_cast<S*>(B0);
    const long nk = (long)nr * M, nb = (long)nr * Dk * M, nx = (long)nr * D, ng = (long)nr * Dk;
    const long ob = (long)RG * M, ox = ob + (long)RG * Dk * M, om = ox + (long)RG * D, ov = om + (long)RG * Dk;
    for (long e = tid; e < nk + nb + nx + 2 * ng; e += nth) {
      long o;
      const S* src;
      if (e < nk) {
        o = e;
        src = (dkfu ? dkfu : kfu) + (size_t)n0 * M + e;
      } else if (e < nk + nb) {
        o = ob + (e - nk);
        src = Bk + (size_t)n0 * Dk * M + (e - nk);
      } else if (e < nk + nb + nx) {
        const long t = e - nk - nb, r = t / D;
        o = ox + t;
        src = x + (size_t)(n0 + r) * ldx + (t - r * D);
      } else if (e < nk + nb + nx + ng) {
        o = om + (e - nk - nb - nx);
        src = dm + (size_t)n0 * Dk + (e - nk - nb - nx);
      } else {
        o = ov + (e - nk - nb - nx - ng);
        src = dv + (size_t)n0 * Dk + (e - nk - nb - nx - ng);
      }
      o = GPK_IDX(o, BS, 4);
      if (convert) {
        B0[o] = Num<T>::ld(R0[o]);
      } else {
        const unsigned d = (unsigned)__cvta_generic_to_shared(R0 + o);
        if (sizeof(S) == 8)
          asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src));
        else
          asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src));
      }
    }
  };
  // Z and A the same way (with the first pass's rows)
  auto zabuf = [&](bool convert) {
    S* zr = reinterpret_cast<S*>(zs);
    for (long e = tid; e < (long)M * D + (long)Dk * M; e += nth) {
      const S* src = e < (long)M * D ? z + e : A + (e - (long)M * D);
      if (convert) {
        zs[e] = Num<T>::ld(zr[e]);
      } else {
        const unsigned d = (unsigned)__cvta_generic_to_shared(zr + e);
        if (sizeof(S) == 8)
          asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src));
        else
          asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src));
      }
    }
  };
  zabuf(false);
  if (nbeg < nend) rowbuf(0, nbeg, min(RG, nend - nbeg), false);
  load_exp_table(tab);
  __syncthreads();
  load_hyp(*h, lls2, lsf2, D, tab);
  asm volatile("cp.async.wait_all;\n" ::: "memory");
  zabuf(true);
  if (nbeg < nend) rowbuf(0, nbeg, min(RG, nend - nbeg), true);
  __syncthreads();
  T zb[DC], gz[DC], gl[DC];
#pragma unroll
  for (int q = 0; q < DC; ++q) {
    zb[q] = (b < M && q < D) ? zs[b * D + q] : Num<T>::zero();
    gz[q] = gl[q] = Num<T>::zero();
  }
  T ab[DO_MAX], ga[DO_MAX];
#pragma unroll
  for (int d = 0; d < DO_MAX; ++d) {
    ab[d] = (b < M && d < Dk) ? as[d * M + b] : Num<T>::zero();
    ga[d] = Num<T>::zero();
  }
  T gsf = Num<T>::zero();
  auto q_on = [&](int q) { return EX || q < D; };
  auto d_on = [&](int d) { return d < DB && (DB < DO_MAX || d < Dout); };
  for (int n0 = nbeg, it = 0; n0 < nend; n0 += RG, ++it) {
    const int n = n0 + rg;
    const bool row = n < nend;
    const int nr = min(RG, nend - n0);
    const bool more = n0 + RG < nend;
    if (more) rowbuf(it + 1, n0 + RG, min(RG, nend - n0 - RG), false);   // the next pass's rows
    const T* B0 = buf + (size_t)(it & 1) * BS;
    const T* kr = B0 + (size_t)rg * M;
    const T* bkr = B0 + (size_t)RG * M + (size_t)rg * Dk * M;
    const T* xs = B0 + (size_t)RG * M * (1 + Dk) + (size_t)rg * D;
    const T* dmr = B0 + (size_t)RG * (M * (1 + Dk) + D) + (size_t)rg * Dk;
    const T* dvr = dmr + (size_t)RG * Dk;
    T L = Num<T>::zero();
    if (row && b < M) {
      const T k = kr[b];
      T g = Num<T>::zero();
      if (dkfu) {
        g = k;   // the staged row holds dkfu here
      } else {
#pragma unroll
        for (int d = 0; d < DB; ++d) {
          if (d_on(d)) {
            const T dmd = dmr[d], dvd = dvr[d];
            g = fma_(dmd, ab[d], g);
            g = fma_(scale2(dvd, 1), bkr[(size_t)d * M + b], g);
            ga[d] = fma_(dmd, k, ga[d]);
          }
        }
      }
      const T kk = dkfu ? Num<T>::ld(kfu[(size_t)n * M + b]) : k;
      L = mul(g, kk);
      gsf = add(gsf, L);
#pragma unroll
      for (int q = 0; q < DC; ++q) {
        if (q_on(q)) {
          const T df = sub(xs[q], zb[q]);
          const T t = mul(L, df);
          gz[q] = fma_(t, h->inv_l2[q], gz[q]);
          gl[q] = fma_(t, df, gl[q]);
        }
      }
    }
    if (dx) {
      // dx_nq = -sum_b L (x_nq - z_bq) / l_q: warp sums over b (all q in one butterfly), then
      // over the group's warps
#pragma unroll
      for (int c0 = 0; c0 < DC; c0 += 8) {   // eight dimensions per butterfly (register budget)
        T t[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int q = c0 + u;
          t[u] = (q_on(q) && row && b < M) ? mul(L, mul(sub(xs[q], zb[q]), h->inv_l2[q])) : Num<T>::zero();
        }
        warp_sum_many<8>(t);   // lane l now holds the warp total of dimension c0 + l / 4
        const int q = c0 + (lane >> 2);
        if ((lane & 3) == 0 && q < D) red[(rg * XW + xw) * DC + q] = t[0];
      }
      __syncthreads();
      if (row && b < D) {
        T sacc = Num<T>::zero();
        for (int w = 0; w < XW; ++w) sacc = add(sacc, red[(rg * XW + w) * DC + b]);
        dx[(size_t)n * D + b] = Num<T>::st(neg(sacc));
      }
    }
    (void)nr;
    if (more) {   // the next pass's rows: this thread's copies landed; convert them, publish
      asm volatile("cp.async.wait_all;\n" ::: "memory");
      rowbuf(it + 1, n0 + RG, min(RG, nend - n0 - RG), true);
    }
    __syncthreads();
  }
  // per-b sums over the row groups -> one write per CTA and (b, q) / (d, b): into this CTA's
  // partial block ([dZ M*D | dA Dout*M | dsf2 | dl D], fixed-order path) or atomically
  double* const pblk = part ? part + (size_t)blockIdx.x * part_stride : nullptr;
  T* pb = red;   // [RG][blockDim.x][DC + DO_MAX]
  const int W = DC + DO_MAX;
#pragma unroll
  for (int q = 0; q < DC; ++q) pb[(rg * blockDim.x + b) * W + q] = gz[q];
#pragma unroll
  for (int d = 0; d < DO_MAX; ++d) pb[(rg * blockDim.x + b) * W + DC + d] = ga[d];
  __syncthreads();
  if (rg == 0 && b < M) {
#pragma unroll
    for (int q = 0; q < DC; ++q) {
      if (q < D) {
        T sacc = pb[b * W + q];
        for (int r = 1; r < RG; ++r) sacc = add(sacc, pb[(r * blockDim.x + b) * W + q]);
        if (pblk) pblk[(size_t)b * D + q] = (double)Num<T>::st(sacc);
        else atomicAdd(&dZ[(size_t)b * D + q], (double)Num<T>::st(sacc));
      }
    }
    const bool wantA = dA && !dkfu;
#pragma unroll
    for (int d = 0; d < DO_MAX; ++d) {
      if (d < (dkfu ? 0 : Dout)) {
        T sacc = pb[b * W + DC + d];
        for (int r = 1; r < RG; ++r) sacc = add(sacc, pb[(r * blockDim.x + b) * W + DC + d]);
        if (pblk) pblk[(size_t)M * D + (size_t)d * M + b] = wantA ? (double)Num<T>::st(sacc) : 0.0;
        else if (wantA) atomicAdd(&dA[(size_t)d * M + b], (double)Num<T>::st(sacc));
      }
    }
  }
  __syncthreads();
  // dsf2 and dl: CTA reduction (the 1 + D warp sums in one butterfly, then lane i of warp 0
  // adds value i over the warps in order)
  const int wid = tid >> 5, nw = nth >> 5, ln = tid & 31;
  T* rw = red;   // [nw][1 + DC]
#pragma unroll
  for (int c0 = 0; c0 < 1 + DC; c0 += 8) {   // values 0 (sf2) and 1 + q (dimension q), eight at a time
    T vals[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int i = c0 + u;
      vals[u] = i == 0 ? gsf : (i <= DC ? gl[(i - 1) & (DC - 1)] : Num<T>::zero());
    }
    warp_sum_many<8>(vals);
    const int i = c0 + (ln >> 2);
    if ((ln & 3) == 0 && i < 1 + DC) rw[wid * (1 + DC) + i] = vals[0];
  }
  __syncthreads();
  if (wid == 0 && ln < 1 + DC) {
    T tot = rw[ln];
    for (int w = 1; w < nw; ++w) tot = add(tot, rw[w * (1 + DC) + ln]);
    const size_t o = (size_t)M * D + (size_t)(dkfu ? 0 : Dout) * M;
    if (ln == 0) {
      const double vsf = (double)Num<T>::st(div(tot, h->sf2));
      if (pblk) pblk[o] = vsf;
      else atomicAdd(dsf2, vsf);
    } else if (ln - 1 < D) {
      // d/d ell of exp(-(x-z)^2/(2 ell^2)) = (x-z)^2 / ell^3 = (x-z)^2 * (1/l)^{3/2}
      const int q = ln - 1;
      const T il = h->inv_l2[q];
      const double vl = (double)Num<T>::st(mul(tot, mul(il, sqrt_(il))));
      if (pblk) pblk[o + 1 + q] = vl;
      else atomicAdd(&dl[q], vl);
    }
  }
}

// Weighted Gram reduction:  C[d] += sum_n w[n,d] u_n v_n^T  (u, v: [N,M] rows; C: [Dout,M,M] f64)
// 32x32 output tile per CTA, n split across gridDim.z.  Rows are staged GB at a time, with
// all of a stage's global loads in flight together.  (The dBhat / dSucav einsums of
// geepee/aep_models.py:463-464, 490-493.)
constexpr int GB = 32;
template <typename T>
__global__ void __launch_bounds__(256) gram_kernel(int N, int M, int Dout, const typename Num<T>::store_t* u,
                                                   const typename Num<T>::store_t* v,
                                                   const typename Num<T>::store_t* w, double* C, int sym,
                                                   double* part) {
  typedef typename Num<T>::store_t S;
  __shared__ T su[GB][32], sv[GB][32], sw[GB][DO_MAX];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 8 rows of threads, 4 outputs each
  // sym (u == v, C symmetric): blockIdx.x enumerates the tiles bi <= bj only, and an
  // off-diagonal tile is added at both (i, j) and (j, i)
  int bi = blockIdx.y, bj = blockIdx.x;
  if (sym) {
    const int nt = (M + 31) >> 5;
    bi = 0;
    bj = blockIdx.x;
    while (bj >= nt - bi) {
      bj -= nt - bi;
      ++bi;
    }
    bj += bi;
  }
  const int i0 = bi * 32, j0 = bj * 32;
  T acc[DO_MAX][4];
#pragma unroll
  for (int d = 0; d < DO_MAX; ++d)
#pragma unroll
    for (int r = 0; r < 4; ++r) acc[d][r] = Num<T>::zero();
  const int nbeg = (int)((long)N * blockIdx.z / gridDim.z), nend = (int)((long)N * (blockIdx.z + 1) / gridDim.z);
  for (int n0 = nbeg; n0 < nend; n0 += GB) {
    // stage rows n0 .. n0+GB-1: element e = tid + 256 p of the u and v tiles (row e/32, col e%32)
    S ru[4], rv[4], rw = S(0);
#pragma unroll
    for (int p = 0; p < 4; ++p) {
      const int e = threadIdx.x + 256 * p, rl = e >> 5, c = e & 31, n = n0 + rl;
      ru[p] = (n < nend && i0 + c < M) ? u[(size_t)n * M + i0 + c] : S(0);
      rv[p] = (n < nend && j0 + c < M) ? v[(size_t)n * M + j0 + c] : S(0);
    }
    {
      const int rl = threadIdx.x / DO_MAX, d = threadIdx.x % DO_MAX, n = n0 + rl;
      if (rl < GB && d < Dout && n < nend) rw = w[(size_t)n * Dout + d];
    }
#pragma unroll
    for (int p = 0; p < 4; ++p) {
      const int e = threadIdx.x + 256 * p;
      su[e >> 5][e & 31] = Num<T>::ld(ru[p]);
      sv[e >> 5][e & 31] = Num<T>::ld(rv[p]);
    }
    if (threadIdx.x < GB * DO_MAX) sw[threadIdx.x / DO_MAX][threadIdx.x % DO_MAX] = Num<T>::ld(rw);
    __syncthreads();
    const int nr = min(GB, nend - n0);
    for (int rl = 0; rl < nr; ++rl) {
      const T vj = sv[rl][tx];
#pragma unroll
      for (int d = 0; d < DO_MAX; ++d) {
        if (d < Dout) {
          const T wv = mul(sw[rl][d], vj);
#pragma unroll
          for (int r = 0; r < 4; ++r) acc[d][r] = fma_(su[rl][ty * 4 + r], wv, acc[d][r]);
        }
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int d = 0; d < DO_MAX; ++d) {
    if (d < Dout) {
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        int i = i0 + ty * 4 + r, j = j0 + tx;
        if (i < M && j < M) {
          const double val = (double)Num<T>::st(acc[d][r]);
          if (part) {   // fixed-order path: this row chunk's partial matrices, plain stores
            double* pc = part + (size_t)blockIdx.z * Dout * M * M;
            pc[((size_t)d * M + i) * M + j] = val;
            if (sym && bi != bj) pc[((size_t)d * M + j) * M + i] = val;
          } else {
            atomicAdd(&C[((size_t)d * M + i) * M + j], val);
            if (sym && bi != bj) atomicAdd(&C[((size_t)d * M + j) * M + i], val);
          }
        }
      }
    }
  }
}

// Symmetric weighted Gram reduction by unordered pairs:  C[d] += sum_n w[n,d] u_n u_n^T
// (the dBhat einsum of geepee/aep_models.py:463-464 with u = kfu).  A CTA owns GP_PPT pairs
// (a >= b, row-major lower-triangle order) per thread of one pair block and one chunk of rows
// (blockIdx.y); the chunk's rows go through shared memory GR at a time, and each pair's sum
// over the chunk is one product u_a u_b per row and one multiply-add per output.  Every pair is
// computed once (no tile padding, no lower half of diagonal tiles); the chunk's sums leave as a
// partial block of packed pairs for the fixed-order reduction.
constexpr int GP_PPT = 2;
constexpr int GP_T = 512;
template <typename T, int DB>
__global__ void __launch_bounds__(GP_T) gram_pairs_kernel(int N, int M, int Dout, const typename Num<T>::store_t* u,
                                                          const typename Num<T>::store_t* w, double* part,
                                                          long pstride, int GR) {
  typedef typename Num<T>::store_t S;
  extern __shared__ __align__(16) char smem_raw[];
  T* us = reinterpret_cast<T*>(smem_raw);   // [GR][M]
  T* ws = us + (size_t)GR * M;              // [GR][DO_MAX]
  const int tid = threadIdx.x, P = M * (M + 1) / 2;
  int ia[GP_PPT], ib[GP_PPT], pp[GP_PPT];
#pragma unroll
  for (int k = 0; k < GP_PPT; ++k) {
    pp[k] = blockIdx.x * (GP_T * GP_PPT) + tid + GP_T * k;
    tri_pair(pp[k] < P ? pp[k] : 0, ia[k], ib[k]);   // pairs past P compute (0, 0), never stored
  }
  // DB (compile-time) outputs per pair, so that the loop below has no branch between the
  // independent sums (DB = 4 serves Dout = 3 with a zero weight)
  T acc[GP_PPT][DB];
#pragma unroll
  for (int k = 0; k < GP_PPT; ++k)
#pragma unroll
    for (int d = 0; d < DB; ++d) acc[k][d] = Num<T>::zero();
  const int nbeg = (int)((long)N * blockIdx.y / gridDim.y), nend = (int)((long)N * (blockIdx.y + 1) / gridDim.y);
  for (int n0 = nbeg; n0 < nend; n0 += GR) {
    const int nr = min(GR, nend - n0);
    stage_async(reinterpret_cast<S*>(us), u + (size_t)n0 * M, (long)nr * M, tid, GP_T);
    for (int e = tid; e < nr * DO_MAX; e += GP_T) {
      const int r = e / DO_MAX, d = e - r * DO_MAX;
      ws[e] = d < Dout ? Num<T>::ld(w[(size_t)(n0 + r) * Dout + d]) : Num<T>::zero();
    }
    __syncthreads();
    convert_in_place(us, (long)nr * M, tid, GP_T);
    __syncthreads();
    for (int rl = 0; rl < nr; ++rl) {
      const T* ur = us + (size_t)rl * M;
      T wd[DB];
#pragma unroll
      for (int d = 0; d < DB; ++d) wd[d] = ld_al8(ws + rl * DO_MAX + d);
#pragma unroll
      for (int k = 0; k < GP_PPT; ++k) {
        const T kk = mul(ld_al8(ur + ia[k]), ld_al8(ur + ib[k]));
#pragma unroll
        for (int d = 0; d < DB; ++d) acc[k][d] = fma_(wd[d], kk, acc[k][d]);
      }
    }
    __syncthreads();   // the rows are consumed before the next chunk overwrites them
  }
  double* pb = part + (size_t)blockIdx.y * pstride;
#pragma unroll
  for (int k = 0; k < GP_PPT; ++k) {
    if (pp[k] < P) {
#pragma unroll
      for (int d = 0; d < DB; ++d)
        if (d < Dout) pb[(size_t)d * P + pp[k]] = (double)Num<T>::st(acc[k][d]);
    }
  }
}

// c[d] += sum_n w[n,d] u_n  (u: [N,M]; c: [Dout,M] f64).  32 columns per CTA, rows split over
// 8 warps and gridDim.y; each thread keeps WU rows' loads in flight at a time.
constexpr int WU = 4;
template <typename T>
__global__ void __launch_bounds__(256) wsum_kernel(int N, int M, int Dout, const typename Num<T>::store_t* u,
                                                   const typename Num<T>::store_t* w, double* c) {
  typedef typename Num<T>::store_t S;
  const int j = blockIdx.x * 32 + (threadIdx.x & 31);
  const int part = threadIdx.x >> 5;  // 8 n-partitions per CTA
  __shared__ T red[8][32][DO_MAX];
  T acc[DO_MAX];
#pragma unroll
  for (int d = 0; d < DO_MAX; ++d) acc[d] = Num<T>::zero();
  const int stride = gridDim.y * 8;
  if (j < M) {
    for (int n0 = blockIdx.y * 8 + part; n0 < N; n0 += stride * WU) {
      S ru[WU], rw[WU][DO_MAX];
#pragma unroll
      for (int t = 0; t < WU; ++t) {
        const int n = n0 + t * stride;
        ru[t] = n < N ? u[(size_t)n * M + j] : S(0);
#pragma unroll
        for (int d = 0; d < DO_MAX; ++d) rw[t][d] = (n < N && d < Dout) ? w[(size_t)n * Dout + d] : S(0);
      }
#pragma unroll
      for (int t = 0; t < WU; ++t) {
        const T uv = Num<T>::ld(ru[t]);
#pragma unroll
        for (int d = 0; d < DO_MAX; ++d)
          if (d < Dout) acc[d] = fma_(Num<T>::ld(rw[t][d]), uv, acc[d]);
      }
    }
  }
#pragma unroll
  for (int d = 0; d < DO_MAX; ++d) red[part][threadIdx.x & 31][d] = acc[d];
  __syncthreads();
  if (part == 0 && j < M) {
    for (int d = 0; d < Dout && d < DO_MAX; ++d) {
      T s = red[0][threadIdx.x][d];
      for (int p = 1; p < 8; ++p) s = add(s, red[p][threadIdx.x][d]);
      atomicAdd(&c[(size_t)d * M + j], (double)Num<T>::st(s));
    }
  }
}

size_t det_fwd_smem(int M, int D, bool zstage, size_t tsz) {
  return 256 * 8 + sizeof(Hyp<df64>) + ((size_t)FT * M + FKA * FCB + 8 * DO_MAX * FT + FT * D + (zstage ? (size_t)M * D : 0)) * tsz;
}
size_t det_bwd_smem(int bx, int rg, int dc, int M, int D, int Dk, size_t tsz) {
  const size_t red = (size_t)rg * bx * (dc + DO_MAX);   // the largest of the three uses of the area
  return 256 * 8 + sizeof(Hyp<df64>) +
         ((size_t)M * D + (size_t)Dk * M + 2 * (size_t)det_bwd_rowbuf(rg, M, D, Dk) + red) * tsz;
}

template <typename T>
int kern_launch(int N, int M, int D, const void* x, int ldx, const void* z, int ldz, const double* lls2,
                const double* lsf2, double jitter, void* K, int ldk, cudaStream_t st) {
  typedef typename Num<T>::store_t S;
  const dim3 grid(gpk::ceil_div(M, KC), gpk::ceil_div(N, KR));
  GPK_REQUIRE(grid.y <= 65535, "kern: N=%d too large (at most %d rows)", N, 65535 * KR);
  const size_t sm = 256 * sizeof(float2) + sizeof(Hyp<T>) + (size_t)(KR + KC) * D * sizeof(T);
  auto k = kern_matrix_kernel<T>;
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k<<<grid, 256, sm, st>>>(N, M, D, (const S*)x, ldx, (const S*)z, ldz, lls2, lsf2, jitter, (S*)K, ldk);
  return gpk::check_launch("kern");
}

}  // namespace

extern "C" int gpk_kern(int prec, int N, int M, int D, const void* x, int ldx, const void* z, int ldz,
                        const double* lls2, const double* lsf2, double jitter, void* K, int ldk, void* stream) {
  GPK_NVTX("gpk_kern");
  GPK_REQUIRE(N >= 0 && M >= 0 && D >= 1 && D <= DMAXK, "kern: bad sizes N=%d M=%d D=%d", N, M, D);
  GPK_REQUIRE(x && z && lls2 && lsf2 && K, "kern: null pointer");
  GPK_REQUIRE(ldx >= D && ldz >= D && ldk >= M, "kern: bad leading dimension");
  if (N == 0 || M == 0) return GPK_OK;
  cudaStream_t st = gpk::as_stream(stream);
  if (prec == GPK_DF64) return kern_launch<df64>(N, M, D, x, ldx, z, ldz, lls2, lsf2, jitter, K, ldk, st);
  if (prec == GPK_FP32) return kern_launch<float>(N, M, D, x, ldx, z, ldz, lls2, lsf2, jitter, K, ldk, st);
  return gpk::fail(GPK_EINVAL, "kern: unknown precision %d", prec);
}

extern "C" int gpk_det_fwd(int prec, int N, int M, int D, int Dout, const void* x, int ldx, const void* Z,
                           const double* lls2, const double* lsf2, const void* A, const void* B, void* kfu,
                           void* Bk, void* m_out, void* v_out, void* stream) {
  GPK_NVTX("gpk_det_fwd");
  GPK_REQUIRE(N >= 0 && M >= 1 && M <= 1024 && D >= 1 && D <= DMAXK, "det_fwd: bad sizes N=%d M=%d D=%d", N, M, D);
  GPK_REQUIRE(Dout >= 1 && Dout <= DO_MAX, "det_fwd: Dout=%d outside [1,%d]", Dout, DO_MAX);
  GPK_REQUIRE(x && Z && lls2 && lsf2 && A && B, "det_fwd: null input");
  if (N == 0) return GPK_OK;
  cudaStream_t st = gpk::as_stream(stream);
  // one CTA column per output d; row tiles up to two resident CTAs per SM in all
  int gx = gpk::ceil_div(N, FT);
  const int cap = std::max(1, gpk::sm_count() * 2 / Dout);
  if (gx > cap) gx = cap;
  const dim3 grid(gx, Dout);
  const int zstage = (size_t)M * D * sizeof(df64) <= 32 * 1024;
  if (prec == GPK_DF64) {
    size_t sm = det_fwd_smem(M, D, zstage, sizeof(df64));
    auto k = det_fwd_kernel<df64>;
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k<<<grid, 256, sm, st>>>(N, M, D, Dout, (const double*)x, ldx, (const double*)Z, lls2, lsf2,
                             (const double*)A, (const double*)B, (double*)kfu, (double*)Bk, (double*)m_out,
                             (double*)v_out, zstage);
  } else if (prec == GPK_FP32) {
    size_t sm = det_fwd_smem(M, D, zstage, sizeof(float));
    auto k = det_fwd_kernel<float>;
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k<<<grid, 256, sm, st>>>(N, M, D, Dout, (const float*)x, ldx, (const float*)Z, lls2, lsf2, (const float*)A,
                             (const float*)B, (float*)kfu, (float*)Bk, (float*)m_out, (float*)v_out, zstage);
  } else {
    return gpk::fail(GPK_EINVAL, "det_fwd: unknown precision %d", prec);
  }
  return gpk::check_launch("det_fwd");
}

namespace {
template <typename T, int DB>
void contract_launch(int N, int M, int Dout, const void* kfu, const double* lsf2, const void* A, const void* B,
                     int b_pairs, void* Bk, void* m_out, void* v_out, cudaStream_t st) {
  typedef typename Num<T>::store_t S;
  const size_t sm = det_contract_smem(M, Dout, sizeof(T));
  auto k = det_contract_kernel<T, DB>;
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k<<<gpk::ceil_div(N, CR), CT, sm, st>>>(N, M, Dout, (const S*)kfu, lsf2, (const S*)A, (const S*)B, (S*)Bk,
                                          (S*)m_out, (S*)v_out, b_pairs);
}
template <typename T>
void contract_dispatch(int N, int M, int Dout, const void* kfu, const double* lsf2, const void* A, const void* B,
                       int b_pairs, void* Bk, void* m_out, void* v_out, cudaStream_t st) {
  if (Dout == 1) contract_launch<T, 1>(N, M, Dout, kfu, lsf2, A, B, b_pairs, Bk, m_out, v_out, st);
  else if (Dout == 2) contract_launch<T, 2>(N, M, Dout, kfu, lsf2, A, B, b_pairs, Bk, m_out, v_out, st);
  else contract_launch<T, 4>(N, M, Dout, kfu, lsf2, A, B, b_pairs, Bk, m_out, v_out, st);
}
}  // namespace

extern "C" int gpk_det_contract_supported(int prec, int M, int Dout) {
  const size_t tsz = prec == GPK_FP32 ? sizeof(float) : sizeof(df64);
  return M >= 1 && M <= 128 && Dout >= 1 && Dout <= DO_MAX && det_contract_smem(M, Dout, tsz) <= 227 * 1024;
}

extern "C" int gpk_det_contract(int prec, int N, int M, int Dout, const void* kfu, const double* lsf2, const void* A,
                                const void* B, int b_pairs, void* Bk, void* m_out, void* v_out, void* stream) {
  GPK_NVTX("gpk_det_contract");
  GPK_REQUIRE(prec == GPK_DF64 || prec == GPK_FP32, "det_contract: unknown precision %d", prec);
  GPK_REQUIRE(!b_pairs || prec == GPK_DF64, "det_contract: double-float pairs need GPK_DF64");
  GPK_REQUIRE(N >= 0 && M >= 1 && Dout >= 1, "det_contract: bad sizes N=%d M=%d Dout=%d", N, M, Dout);
  if (!gpk_det_contract_supported(prec, M, Dout))
    return gpk::fail(GPK_EUNSUPPORTED, "det_contract: M=%d, Dout=%d (needs M <= 128 and Dout M^2 in shared memory)",
                     M, Dout);
  GPK_REQUIRE(kfu && lsf2 && A && B, "det_contract: null input");
  if (N == 0) return GPK_OK;
  cudaStream_t st = gpk::as_stream(stream);
  if (prec == GPK_DF64) contract_dispatch<df64>(N, M, Dout, kfu, lsf2, A, B, b_pairs, Bk, m_out, v_out, st);
  else contract_dispatch<float>(N, M, Dout, kfu, lsf2, A, B, 0, Bk, m_out, v_out, st);
  return gpk::check_launch("det_contract");
}

extern "C" int gpk_det_bwd(int prec, int N, int M, int D, int Dout, const void* x, int ldx, const void* Z,
                           const double* lls2, const double* lsf2, const void* A, const void* kfu, const void* Bk,
                           const void* dm, const void* dv, const void* dkfu, double* dsf2, double* dl, double* dZ,
                           double* dA, void* dx, void* stream) {
  GPK_NVTX("gpk_det_bwd");
  return gpk_det_bwd_ws(prec, N, M, D, Dout, x, ldx, Z, lls2, lsf2, A, kfu, Bk, dm, dv, dkfu, dsf2, dl, dZ, dA, dx,
                        nullptr, 0, stream);
}

namespace {
// rows split over CTAs: threads are b (a multiple of 32 >= M) x row groups, 512 at most; CTAs of
// two passes of the row groups (8 rows at rg = 4): 125 CTAs for 1000 rows, one per SM at most
int det_bwd_grid(int N, int M) {
  const int bx = 32 * gpk::ceil_div(M, 32), rg = bx <= 128 ? 4 : 2;
  int grid = gpk::ceil_div(N, 2 * rg);
  if (grid > gpk::sm_count()) grid = gpk::sm_count();
  return grid;
}
long det_bwd_stride(int M, int D, int Dout, bool dkfu) { return (long)M * D + (long)(dkfu ? 0 : Dout) * M + 1 + D; }

// gram: 32 x 32 output tiles (the upper ones only when C is symmetric), rows split over
// gridDim.z chunks so that about two CTAs run per SM
int gram_chunks(int N, int M, bool sym) {
  const int nt = gpk::ceil_div(M, 32);
  const int tiles = sym ? nt * (nt + 1) / 2 : nt * nt;
  int chunks = gpk::ceil_div(gpk::sm_count() * 2, tiles);
  if (chunks > gpk::ceil_div(N, 16)) chunks = gpk::ceil_div(N, 16);
  if (chunks < 1) chunks = 1;
  return chunks;
}
}  // namespace

namespace {
template <typename T, int DC, int DB, bool EX>
void det_bwd_launch(int grid, dim3 threads, cudaStream_t st, int N, int M, int D, int Dout, const void* x, int ldx,
                    const void* Z, const double* lls2, const double* lsf2, const void* A, const void* kfu,
                    const void* Bk, const void* dm, const void* dv, const void* dkfu, double* dsf2, double* dl,
                    double* dZ, double* dA, void* dx, double* work, long stride) {
  typedef typename Num<T>::store_t S;
  const size_t sm = det_bwd_smem(threads.x, threads.y, DC, M, D, dkfu ? 0 : Dout, sizeof(T));
  auto k = det_bwd_kernel<T, DC, DB, EX>;
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k<<<grid, threads, sm, st>>>(N, M, D, Dout, (const S*)x, ldx, (const S*)Z, lls2, lsf2, (const S*)A, (const S*)kfu,
                               (const S*)Bk, (const S*)dm, (const S*)dv, (const S*)dkfu, dsf2, dl, dZ, dA, (S*)dx,
                               work, stride);
}
// the exact forms for D = 8 inputs and 1 or 2 outputs given through A, Bk (the deep GP's first
// layer and the 8-input regressions); everything else takes the general form
template <typename T>
void det_bwd_dispatch(int grid, dim3 threads, cudaStream_t st, int dc, int N, int M, int D, int Dout, const void* x,
                      int ldx, const void* Z, const double* lls2, const double* lsf2, const void* A, const void* kfu,
                      const void* Bk, const void* dm, const void* dv, const void* dkfu, double* dsf2, double* dl,
                      double* dZ, double* dA, void* dx, double* work, long stride) {
#define GPK_DET_BWD_ARGS grid, threads, st, N, M, D, Dout, x, ldx, Z, lls2, lsf2, A, kfu, Bk, dm, dv, dkfu, dsf2, dl, \
                         dZ, dA, dx, work, stride
  if (D == 8 && !dkfu && Dout == 1) det_bwd_launch<T, 8, 1, true>(GPK_DET_BWD_ARGS);
  else if (D == 8 && !dkfu && Dout == 2) det_bwd_launch<T, 8, 2, true>(GPK_DET_BWD_ARGS);
  else if (dc == 8) det_bwd_launch<T, 8, DO_MAX, false>(GPK_DET_BWD_ARGS);
  else det_bwd_launch<T, 16, DO_MAX, false>(GPK_DET_BWD_ARGS);
#undef GPK_DET_BWD_ARGS
}
}  // namespace

long det_bwd_work_elems(int N, int M, int D, int Dout) {
  return (long)gpk::sm_count() * det_bwd_stride(M, D, Dout, false);
}
namespace {
// the pair-wise Gram reduction: pair blocks of GP_T * GP_PPT pairs, row chunks so that about one
// CTA runs per SM, each chunk at least 8 rows; rows staged GR at a time (about 48 KB)
int gram_pair_blocks(int M) { return gpk::ceil_div(M * (M + 1) / 2, GP_T * GP_PPT); }
int gram_pair_chunks(int N, int M) {
  int c = gpk::ceil_div(gpk::sm_count(), gram_pair_blocks(M));
  const int cap = gpk::ceil_div(N, 8);
  if (c > cap) c = cap;
  return c < 1 ? 1 : c;
}
template <typename T, int DB>
void gram_pairs_launch(dim3 grid, size_t sm, cudaStream_t st, int N, int M, int Dout, const void* u, const void* w,
                       double* work, long pstride, int GR) {
  typedef typename Num<T>::store_t S;
  auto k = gram_pairs_kernel<T, DB>;
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k<<<grid, GP_T, sm, st>>>(N, M, Dout, (const S*)u, (const S*)w, work, pstride, GR);
}
template <typename T>
void gram_pairs_dispatch(dim3 grid, size_t sm, cudaStream_t st, int N, int M, int Dout, const void* u, const void* w,
                         double* work, long pstride, int GR) {
  if (Dout == 1) gram_pairs_launch<T, 1>(grid, sm, st, N, M, Dout, u, w, work, pstride, GR);
  else if (Dout == 2) gram_pairs_launch<T, 2>(grid, sm, st, N, M, Dout, u, w, work, pstride, GR);
  else gram_pairs_launch<T, 4>(grid, sm, st, N, M, Dout, u, w, work, pstride, GR);
}

int gram_pair_rows(int M, size_t tsz) {
  const int r = (int)((48 * 1024) / ((size_t)M * tsz + DO_MAX * tsz));
  return r < 1 ? 1 : (r > 32 ? 32 : r);
}
}  // namespace

long gram_work_elems(int N, int M, int Dout) {
  const long full = (long)gram_chunks(N, M, false) * Dout * M * M;   // u != v: full tiles
  const long pairs = (long)gram_pair_chunks(N, M) * Dout * (M * (M + 1) / 2);
  return full > pairs ? full : pairs;
}

extern "C" int gpk_det_bwd_ws(int prec, int N, int M, int D, int Dout, const void* x, int ldx, const void* Z,
                              const double* lls2, const double* lsf2, const void* A, const void* kfu, const void* Bk,
                              const void* dm, const void* dv, const void* dkfu, double* dsf2, double* dl, double* dZ,
                              double* dA, void* dx, double* work, long work_elems, void* stream) {
  GPK_NVTX("gpk_det_bwd_ws");
  GPK_REQUIRE(N >= 0 && M >= 1 && M <= 256 && D >= 1 && D <= 16, "det_bwd: bad sizes N=%d M=%d D=%d (M<=256, D<=16)", N, M, D);
  GPK_REQUIRE(dkfu || (Dout >= 1 && Dout <= DO_MAX), "det_bwd: Dout=%d outside [1,%d]", Dout, DO_MAX);
  GPK_REQUIRE(x && Z && lls2 && lsf2 && kfu && dsf2 && dl && dZ, "det_bwd: null");
  GPK_REQUIRE(dkfu || (A && Bk && dm && dv), "det_bwd: need dkfu or (A, Bk, dm, dv)");
  const long stride = det_bwd_stride(M, D, Dout, dkfu != nullptr);
  if (work) {
    const long need = (long)gpk::sm_count() * stride;
    GPK_REQUIRE(work_elems >= need, "det_bwd: workspace of %ld doubles, %ld needed", work_elems, need);
  }
  if (N == 0) return GPK_OK;
  cudaStream_t st = gpk::as_stream(stream);
  const int bx = 32 * gpk::ceil_div(M, 32), rg = bx <= 128 ? 4 : 2;
  const int grid = det_bwd_grid(N, M);
  const dim3 threads(bx, rg);
  const int dc = D <= 8 ? 8 : 16;
  if (prec == GPK_DF64)
    det_bwd_dispatch<df64>(grid, threads, st, dc, N, M, D, Dout, x, ldx, Z, lls2, lsf2, A, kfu, Bk, dm, dv, dkfu,
                           dsf2, dl, dZ, dA, dx, work, stride);
  else if (prec == GPK_FP32)
    det_bwd_dispatch<float>(grid, threads, st, dc, N, M, D, Dout, x, ldx, Z, lls2, lsf2, A, kfu, Bk, dm, dv, dkfu,
                            dsf2, dl, dZ, dA, dx, work, stride);
  else
    return gpk::fail(GPK_EINVAL, "det_bwd: unknown precision %d", prec);
  int rc = gpk::check_launch("det_bwd");
  if (rc != GPK_OK || !work) return rc;
  gpk::RedPlan plan{};
  plan.add(dZ, M * D);
  plan.add(dA, dkfu ? 0 : Dout * M);
  plan.add(dsf2, 1);
  plan.add(dl, D);
  return gpk::reduce_partials(work, grid, plan, st);
}

extern "C" int gpk_gram(int prec, int N, int M, int Dout, const void* u, const void* v, const void* w, double* C,
                        void* stream) {
  GPK_NVTX("gpk_gram");
  return gpk_gram_ws(prec, N, M, Dout, u, v, w, C, nullptr, 0, stream);
}

extern "C" int gpk_gram_ws(int prec, int N, int M, int Dout, const void* u, const void* v, const void* w, double* C,
                           double* work, long work_elems, void* stream) {
  GPK_NVTX("gpk_gram_ws");
  GPK_REQUIRE(N >= 0 && M >= 1 && Dout >= 1 && Dout <= DO_MAX, "gram: bad sizes");
  GPK_REQUIRE(u && v && w && C, "gram: null pointer");
  const int sym = u == v;   // C symmetric: the upper tiles only
  const int P = M * (M + 1) / 2;
  const int chunks = sym ? gram_pair_chunks(N, M) : gram_chunks(N, M, false);
  if (work) {
    const long need = (long)chunks * Dout * (sym ? P : M * M);
    GPK_REQUIRE(work_elems >= need, "gram: workspace of %ld doubles, %ld needed", work_elems, need);
  }
  if (N == 0) return GPK_OK;
  cudaStream_t st = gpk::as_stream(stream);
  if (sym && work) {   // the fixed-order symmetric form: unordered pairs, packed partial blocks
    const size_t tsz = prec == GPK_FP32 ? sizeof(float) : sizeof(df64);
    const int GR = gram_pair_rows(M, tsz);
    const size_t sm = (size_t)GR * (M + DO_MAX) * tsz;
    const dim3 grid(gram_pair_blocks(M), chunks);
    const long pstride = (long)Dout * P;
    if (prec == GPK_DF64) gram_pairs_dispatch<df64>(grid, sm, st, N, M, Dout, u, w, work, pstride, GR);
    else if (prec == GPK_FP32) gram_pairs_dispatch<float>(grid, sm, st, N, M, Dout, u, w, work, pstride, GR);
    else return gpk::fail(GPK_EINVAL, "gram: unknown precision %d", prec);
    int rc = gpk::check_launch("gram_pairs");
    if (rc != GPK_OK) return rc;
    gpk::RedPlan plan{};
    plan.add(C, Dout * P, 1, M);
    return gpk::reduce_partials(work, chunks, plan, st);
  }
  const int nt = gpk::ceil_div(M, 32);
  const int tchunks = gram_chunks(N, M, sym);   // the tiled form (atomic, or u != v)
  const int tiles = sym ? nt * (nt + 1) / 2 : nt * nt;
  const dim3 grid(sym ? tiles : nt, sym ? 1 : nt, tchunks);
  if (prec == GPK_DF64)
    gram_kernel<df64><<<grid, 256, 0, st>>>(N, M, Dout, (const double*)u, (const double*)v, (const double*)w, C,
                                            sym, work);
  else if (prec == GPK_FP32)
    gram_kernel<float><<<grid, 256, 0, st>>>(N, M, Dout, (const float*)u, (const float*)v, (const float*)w, C,
                                             sym, work);
  else
    return gpk::fail(GPK_EINVAL, "gram: unknown precision %d", prec);
  int rc = gpk::check_launch("gram");
  if (rc != GPK_OK || !work) return rc;
  gpk::RedPlan plan{};
  plan.add(C, Dout * M * M);
  return gpk::reduce_partials(work, tchunks, plan, st);
}

extern "C" int gpk_wsum(int prec, int N, int M, int Dout, const void* u, const void* w, double* c, void* stream) {
  GPK_NVTX("gpk_wsum");
  GPK_REQUIRE(N >= 0 && M >= 1 && Dout >= 1 && Dout <= DO_MAX, "wsum: bad sizes");
  GPK_REQUIRE(u && w && c, "wsum: null pointer");
  if (N == 0) return GPK_OK;
  cudaStream_t st = gpk::as_stream(stream);
  int gy = gpk::ceil_div(N, 8 * WU);
  if (gy > 128) gy = 128;
  dim3 grid(gpk::ceil_div(M, 32), gy);
  if (prec == GPK_DF64)
    wsum_kernel<df64><<<grid, 256, 0, st>>>(N, M, Dout, (const double*)u, (const double*)w, c);
  else if (prec == GPK_FP32)
    wsum_kernel<float><<<grid, 256, 0, st>>>(N, M, Dout, (const float*)u, (const float*)w, c);
  else
    return gpk::fail(GPK_EINVAL, "wsum: unknown precision %d", prec);
  return gpk::check_launch("wsum");
}

// the translation unit's bounds word (debug build; 0 otherwise)
GPK_BOUNDS_READER(kern)
