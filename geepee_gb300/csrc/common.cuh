// Shared host/device helpers for the libgpk translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>

#include <nvtx3/nvToolsExt.h>

#include "../../include/gpk.h"
#include "df64.cuh"

// Debug build (-DGPK_DEBUG_BOUNDS; build(debug_bounds=True) -> libgpk_debug.so): the hot
// kernels' indexed accesses go through GPK_IDX(i, n, code).  An index outside [0, n) sets bit
// `code` of this translation unit's error word and is replaced by 0 (an element that exists),
// so the kernel completes and the host reads the word (gpk_debug_bounds).  The release build
// compiles the checks away.  Codes: 0 factor L, 1 GEMM tile staging, 2 psi backward pair
// table / L / accumulators, 3 psi forward pair tables, 4 det backward row buffer, 5 det
// contraction B, 6 psi backward row sums.
#ifdef GPK_DEBUG_BOUNDS
static __device__ unsigned int g_gpk_bounds_word;
__device__ __forceinline__ long gpk_idx(long i, long n, int code) {
  if (i >= 0 && i < n) return i;
  atomicOr(&g_gpk_bounds_word, 1u << code);
  return 0;
}
#define GPK_IDX(i, n, code) gpk_idx((long)(i), (long)(n), (code))
// this translation unit's word, cleared after reading (host side)
#define GPK_BOUNDS_READER(name)                                           \
  unsigned gpk_bounds_word_##name() {                                     \
    unsigned w = 0, z = 0;                                                \
    cudaMemcpyFromSymbol(&w, g_gpk_bounds_word, sizeof(w));               \
    cudaMemcpyToSymbol(g_gpk_bounds_word, &z, sizeof(z));                 \
    return w;                                                             \
  }
#else
#define GPK_IDX(i, n, code) (i)
#define GPK_BOUNDS_READER(name) \
  unsigned gpk_bounds_word_##name() { return 0u; }
#endif

namespace gpk {

// per-thread text of the last error (read by gpk_last_error)
extern thread_local char g_err[512];

inline int fail(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  return code;
}

inline int check_launch(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(GPK_ECUDA, "%s: %s", what, cudaGetErrorString(e));
  return GPK_OK;
}

// number of SMs of the current device (cached per device id)
int sm_count();

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

inline int ceil_div(int a, int b) { return (a + b - 1) / b; }

// Fixed-order accumulation.  A kernel of the deterministic path writes its per-CTA partial sums
// to a workspace, part[c * stride + j] for CTA c, instead of adding them into the outputs with
// atomics; reduce_partials then adds sum_c part[c * stride + j] (in a fixed order of c) into
// segment j's destination.  Each destination element has exactly one writer,
// so repeated runs on the same inputs give bit-identical sums.
constexpr int RED_SEGS = 6;
struct RedSeg {
  double* dst;   // null: the segment is skipped
  int len;
  int kind;      // 0: dst[j] += s;  1: len = D M(M+1)/2 packed pairs (a >= b) of D M x M
                 //    matrices, added at (a, b) and, off the diagonal, at (b, a)
  int M;
};
struct RedPlan {
  int nseg;
  RedSeg seg[RED_SEGS];
  long stride() const {
    long s = 0;
    for (int i = 0; i < nseg; ++i) s += seg[i].len;
    return s;
  }
  void add(double* dst, int len, int kind = 0, int M = 0) { seg[nseg++] = RedSeg{dst, len, kind, M}; }
};
// adds the nparts partial blocks of `part` (stride plan.stride()) into the plan's destinations
int reduce_partials(const double* part, int nparts, const RedPlan& plan, cudaStream_t st);

// An NVTX range named after the C-ABI entry point, open for the call's host-side duration
// (argument checks and launches); nvtx3 is header-only and costs a pointer test when no tool
// is attached.
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
};

}  // namespace gpk

#define GPK_NVTX(name) gpk::NvtxRange gpk_nvtx_range_(name)

// workspace (float64 elements) of the fixed-order path of each accumulating entry point
long psi_bwd_work_elems(int M, int Q, int Dout);
long det_bwd_work_elems(int N, int M, int D, int Dout);
long gram_work_elems(int N, int M, int Dout);
long trace_kzz_work_elems(int M, int Q);

// Pair p of the row-major lower triangle, p = a (a + 1) / 2 + b with 0 <= b <= a.
__host__ __device__ __forceinline__ void tri_pair(int p, int& a, int& b) {
  int r = (int)((sqrtf(8.f * (float)p + 1.f) - 1.f) * 0.5f);
  if ((r + 1) * (r + 2) / 2 <= p) ++r;
  if (r * (r + 1) / 2 > p) --r;
  a = r;
  b = p - r * (r + 1) / 2;
}

// Copies n storage-type elements (8 or 4 bytes) from global memory into shared memory with
// asynchronous copies issued by threads tid, tid + nth, ... (all in flight together), then
// waits for this thread's copies; the caller's barrier makes them visible to the CTA.
template <typename S>
__device__ __forceinline__ void stage_async(S* dst, const S* src, long n, int tid, int nth) {
  static_assert(sizeof(S) == 8 || sizeof(S) == 4, "8- or 4-byte elements");
  for (long e = tid; e < n; e += nth) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst + e);
    if (sizeof(S) == 8)
      asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src + e));
    else
      asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src + e));
  }
  asm volatile("cp.async.wait_all;\n" ::: "memory");
}

// Storage type -> compute type in place (the two have the same size), one element per
// thread step; call between barriers.
template <typename T>
__device__ __forceinline__ void convert_in_place(T* buf, long n, int tid, int nth) {
  typedef typename Num<T>::store_t S;
  static_assert(sizeof(S) == sizeof(T), "in-place conversion needs equal sizes");
  S* raw = reinterpret_cast<S*>(buf);
  for (long e = tid; e < n; e += nth) {
    const S x = raw[e];
    buf[e] = Num<T>::ld(x);
  }
}

#define GPK_REQUIRE(cond, ...) \
  do {                          \
    if (!(cond)) return gpk::fail(GPK_EINVAL, __VA_ARGS__); \
  } while (0)

// log-parameterised hyperparameters -> compute type, evaluated on the device
template <typename T, typename Tab>
__device__ __forceinline__ T exp_of_log(const double* p, const Tab& tab) {
  return exp_tab(Num<T>::ld(static_cast<typename Num<T>::store_t>(*p)), tab);
}

// Elements [start, total) step `stride` of one gpk_lincomb_t (float64 arithmetic):
//   out[b,i,j] = sum_t cX[t] X[t][b, i, j or transposed] + sum_r cr[r] u[r][b,i] v[r][b,j]
// (a batch sum adds over b; a batch-broadcast term then enters once).  Shared by the lincomb
// launch and the grouped launch of one dependency level of the algebra.
static __device__ __forceinline__ void lincomb_run(const gpk_lincomb_t& d, long start, long stride) {
  const long per = (long)d.rows * d.cols;
  const long total = d.sum_batch ? per : per * d.batch;
  for (long e = start; e < total; e += stride) {
    const long b0 = d.sum_batch ? 0 : e / per;
    const long r = e - b0 * per;
    const int i = (int)(r / d.cols), j = (int)(r - (long)i * d.cols);
    const long rt = (long)j * d.cols + i;   // transposed element (square only)
    const int bb = d.sum_batch ? 0 : (int)b0, be = d.sum_batch ? d.batch : (int)b0 + 1;
    double acc = 0.0;
    for (int t = 0; t < d.nterm; ++t) {
      const bool once = d.sum_batch && d.sX[t] == 0;
      for (int b = once ? 0 : bb; b < (once ? 1 : be); ++b)
        acc += d.cX[t] * d.X[t][b * d.sX[t] + (d.tX[t] ? rt : r)];
    }
    for (int t = 0; t < d.nrank; ++t) {
      const bool once = d.sum_batch && d.su[t] == 0 && d.sv[t] == 0;
      for (int b = once ? 0 : bb; b < (once ? 1 : be); ++b)
        acc += d.cr[t] * d.u[t][b * d.su[t] + i] * d.v[t][b * d.sv[t] + j];
    }
    d.out[e] = acc;
  }
}

// argument checks of one gpk_lincomb_t (GPK_OK or the error status); `n` gets its element count
static inline int lincomb_check(const gpk_lincomb_t* d, long* n) {
  GPK_REQUIRE(d && d->out, "lincomb: null descriptor or output");
  GPK_REQUIRE(d->batch >= 1 && d->rows >= 0 && d->cols >= 0, "lincomb: bad shape");
  GPK_REQUIRE(d->nterm >= 0 && d->nterm <= GPK_LC_TERMS && d->nrank >= 0 && d->nrank <= GPK_LC_RANK,
              "lincomb: %d dense / %d rank-one terms (max %d / %d)", d->nterm, d->nrank, GPK_LC_TERMS, GPK_LC_RANK);
  for (int t = 0; t < d->nterm; ++t) {
    GPK_REQUIRE(d->X[t], "lincomb: null dense term %d", t);
    GPK_REQUIRE(!d->tX[t] || d->rows == d->cols, "lincomb: transposed term %d needs a square shape", t);
  }
  for (int t = 0; t < d->nrank; ++t) GPK_REQUIRE(d->u[t] && d->v[t], "lincomb: null rank-one term %d", t);
  *n = (long)d->rows * d->cols * (d->sum_batch ? 1 : d->batch);
  return GPK_OK;
}
