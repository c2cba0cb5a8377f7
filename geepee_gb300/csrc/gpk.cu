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

extern "C" int gpk_version(void) {
  GPK_NVTX("gpk_version"); return 1; }
extern "C" const char* gpk_last_error(void) { return gpk::g_err; }

// the other translation units' bounds words (common.cuh, GPK_BOUNDS_READER)
unsigned gpk_bounds_word_algebra();
unsigned gpk_bounds_word_dense();
unsigned gpk_bounds_word_kern();
unsigned gpk_bounds_word_psi_api();
unsigned gpk_bounds_word_psi_bwd_df64();
unsigned gpk_bounds_word_psi_bwd_f32();
unsigned gpk_bounds_word_psi_fwd_df64();
unsigned gpk_bounds_word_psi_fwd_f32();

extern "C" int gpk_debug_bounds(unsigned int* word) {
  GPK_NVTX("gpk_debug_bounds");
  if (!word) return gpk::fail(GPK_EINVAL, "debug_bounds: null output");
  *word = gpk_bounds_word_algebra() | gpk_bounds_word_dense() | gpk_bounds_word_kern() | gpk_bounds_word_psi_api() |
          gpk_bounds_word_psi_bwd_df64() | gpk_bounds_word_psi_bwd_f32() | gpk_bounds_word_psi_fwd_df64() |
          gpk_bounds_word_psi_fwd_f32();
#ifdef GPK_DEBUG_BOUNDS
  return 1;
#else
  return 0;
#endif
}

namespace {

// Eight lanes per output element j: lane l sums the partials c = l, l + 8, ... in order, then
// the eight lane sums combine over a fixed butterfly (both partners compute the same sum, as
// IEEE addition commutes), and lane 0 adds the total into the element's destination.  Plain
// float64 additions: FP64 issues slowly on this GPU, and a compensated sum would cost ~8x
// for ~150 partials whose rounding (~150 ulp at worst) is far below the df64 results' own.
__global__ void __launch_bounds__(256) reduce_partials_kernel(const double* part, int nparts, long stride,
                                                              gpk::RedPlan plan) {
  const long j = (blockIdx.x * (long)blockDim.x + threadIdx.x) >> 3;
  const int l = threadIdx.x & 7;
  double s0 = 0.0, s1 = 0.0;   // two chains, joined in a fixed order
  if (j < stride) {
    int k = l;
    for (; k + 8 < nparts; k += 16) {
      s0 += part[(size_t)k * stride + j];
      s1 += part[(size_t)(k + 8) * stride + j];
    }
    if (k < nparts) s0 += part[(size_t)k * stride + j];
  }
  double s = s0 + s1;
#pragma unroll
  for (int m = 1; m < 8; m <<= 1) s = s + __shfl_xor_sync(0xffffffffu, s, m);
  if (l != 0 || j >= stride) return;
  const double v = s;
  long off = 0;
  for (int i = 0; i < plan.nseg; ++i) {
    const gpk::RedSeg& g = plan.seg[i];
    if (j < off + g.len) {
      if (!g.dst) return;
      const long jj = j - off;
      if (g.kind == 0) {
        g.dst[jj] += v;
      } else {
        const long P = (long)g.M * (g.M + 1) / 2;
        const long d = jj / P;
        int a, b;
        tri_pair((int)(jj - d * P), a, b);
        double* m = g.dst + (size_t)d * g.M * g.M;
        m[(size_t)a * g.M + b] += v;
        if (a != b) m[(size_t)b * g.M + a] += v;
      }
      return;
    }
    off += g.len;
  }
}

}  // namespace

namespace gpk {
int reduce_partials(const double* part, int nparts, const RedPlan& plan, cudaStream_t st) {
  const long stride = plan.stride();
  if (stride == 0 || nparts <= 0) return GPK_OK;
  const long threads = stride * 8;
  reduce_partials_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(part, nparts, stride, plan);
  return check_launch("reduce_partials");
}
}  // namespace gpk

extern "C" int gpk_work_elems(int op, int N, int M, int D, int Dout, long* elems) {
  GPK_NVTX("gpk_work_elems");
  GPK_REQUIRE(elems, "work_elems: null output");
  GPK_REQUIRE(N >= 0 && M >= 1 && D >= 1 && Dout >= 1, "work_elems: bad sizes N=%d M=%d D=%d Dout=%d", N, M, D, Dout);
  switch (op) {
    case GPK_OP_PSI_BWD: *elems = psi_bwd_work_elems(M, D, Dout); return GPK_OK;
    case GPK_OP_DET_BWD: *elems = det_bwd_work_elems(N, M, D, Dout); return GPK_OK;
    case GPK_OP_GRAM: *elems = gram_work_elems(N, M, Dout); return GPK_OK;
    case GPK_OP_TRACE_KZZ: *elems = trace_kzz_work_elems(M, D); return GPK_OK;
    default: return gpk::fail(GPK_EINVAL, "work_elems: unknown operation %d", op);
  }
}
