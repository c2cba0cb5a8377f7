// Library-wide host helpers: version, per-thread error text, device properties.
#include "common.cuh"

namespace gpk {
thread_local char g_err[512] = "";

int sm_count() {
  static int cache[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 148;
  if (cache[dev] == 0) {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 148;
    cache[dev] = n;
  }
  return cache[dev];
}
}  // namespace gpk

extern "C" int gpk_version(void) { return 1; }
extern "C" const char* gpk_last_error(void) { return gpk::g_err; }
