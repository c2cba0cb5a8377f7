// Shared host/device helpers for the libgpk translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>

#include "../../include/gpk.h"
#include "df64.cuh"

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

}  // namespace gpk

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
