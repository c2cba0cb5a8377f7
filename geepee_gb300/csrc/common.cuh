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
