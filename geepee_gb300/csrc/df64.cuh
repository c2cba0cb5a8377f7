// Double-float ("df64") arithmetic on the FP32 pipes of sm_103a.
//
// A value is the unevaluated sum hi + lo of two floats (|lo| <= ulp(hi)/2), giving
// about 48 significant bits.  GB300 issues FP32 FMAs at ~60x its FP64 rate, so the
// error-free transformations below (Knuth two-sum, FMA two-product) buy FP64-class
// accuracy for the ill-conditioned parts of the sparse-GP path at a fraction of the
// cost of native double.  Algorithms: Dekker/Knuth error-free transforms and the
// double-double scheme of Hida, Li & Bailey ("Algorithms for quad-double precision
// floating point arithmetic", ARITH 2001), specialised to float pairs.
//
// The same kernels are instantiated for plain `float`; the overload set below lets
// templated code be written once (add/mul/fma_/exp_/...).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

struct df64 {
  float hi, lo;
};

__host__ __device__ __forceinline__ df64 make_df(float h, float l = 0.f) { df64 r; r.hi = h; r.lo = l; return r; }

// float64 -> (hi, lo): hi = x rounded to float, lo = (x - hi) rounded to float.  Done with
// integer operations on the bit pattern (round-to-nearest-even of the 53-bit significand to
// 24 bits, then the signed remainder normalised to 24 bits): the FP64 pipe, which the plain
// conversion would use, issues ~64x slower than the integer pipes on this part.  Zeros are
// taken directly (lo may come out subnormal); values whose hi would not be a normal float
// (|x| < 2^-126 or >= 2^128, inf, nan) take the FP64 path.
// Kept out of line: inlined, the compiler if-converts the rare branch that calls it and runs
// its FP64 instructions for every conversion.
static __device__ __noinline__ df64 df_from_double_fp64(double x) {
  float h = __double2float_rn(x);
  float l = __double2float_rn(x - (double)h);
  return make_df(h, l);
}
__device__ __forceinline__ df64 df_from_double(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int e = (int)((b >> 52) & 0x7ff);
  if ((b << 1) == 0ull) return make_df(__int_as_float((int)(b >> 32)), 0.f);   // +-0
  if (e < 897 || e > 1150) return df_from_double_fp64(x);   // hi would be subnormal / inf / nan
  const unsigned long long mant = (b & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull;
  unsigned top = (unsigned)(mant >> 29);
  int rem = (int)(mant & 0x1FFFFFFFull);
  if (rem > 0x10000000 || (rem == 0x10000000 && (top & 1u))) {
    top += 1u;
    rem -= 0x20000000;
  }
  int fe = e - 1023 + 127;
  if (top == 0x1000000u) {
    top >>= 1;
    fe += 1;
  }
  const unsigned sign = (unsigned)(b >> 63);
  const float hi = __uint_as_float((sign << 31) | ((unsigned)fe << 23) | (top & 0x7fffffu));
  float lo = 0.f;
  if (rem != 0) {
    unsigned rs = 0u;
    unsigned r = (unsigned)rem;
    if (rem < 0) {
      rs = 1u;
      r = (unsigned)(-rem);
    }
    const int nb = 32 - __clz(r);
    int sh = nb - 24;
    const unsigned ls = (sign ^ rs) << 31;
    const int le0 = e - 1075 + sh + 23 + 127;   // lo's exponent field before rounding
    if (le0 >= 1) {
      unsigned m;
      if (sh > 0) {
        m = r >> sh;
        const unsigned rem2 = r & ((1u << sh) - 1u), half = 1u << (sh - 1);
        if (rem2 > half || (rem2 == half && (m & 1u))) ++m;
        if (m == 0x1000000u) {
          m >>= 1;
          ++sh;
        }
      } else {
        m = r << (-sh);
      }
      const int le = e - 1075 + sh + 23 + 127;
      lo = __uint_as_float(ls | ((unsigned)le << 23) | (m & 0x7fffffu));
    } else {
      // subnormal lo: round the remainder once, straight to the subnormal's precision (a
      // carry into bit 23 gives the smallest normal, which the bit pattern encodes as is)
      const int t = sh + 1 - le0;
      unsigned q = 0u;
      if (t <= 0) {
        q = r << (-t);
      } else if (t < 32) {
        q = r >> t;
        const unsigned rr = r & ((1u << t) - 1u), hf = 1u << (t - 1);
        if (rr > hf || (rr == hf && (q & 1u))) ++q;
      }
      lo = __uint_as_float(ls | q);
    }
  }
  return make_df(hi, lo);
}
__device__ __forceinline__ double df_to_double(df64 a) { return (double)a.hi + (double)a.lo; }

// ---- error-free transforms ----
__device__ __forceinline__ df64 two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return make_df(s, e);
}
__device__ __forceinline__ df64 quick_two_sum(float a, float b) {  // |a| >= |b|
  float s = __fadd_rn(a, b);
  float e = __fsub_rn(b, __fsub_rn(s, a));
  return make_df(s, e);
}
__device__ __forceinline__ df64 two_prod(float a, float b) {
  float p = __fmul_rn(a, b);
  float e = __fmaf_rn(a, b, -p);
  return make_df(p, e);
}

// ---- arithmetic ----
// "sloppy" double-float add (Hida-Li-Bailey): error <= ~2^-47 (|a| + |b|), the same
// shape of bound as an FP64 add; 11 FP32 ops.
__device__ __forceinline__ df64 add(df64 a, df64 b) {
  df64 s = two_sum(a.hi, b.hi);
  s.lo = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
  return quick_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ df64 neg(df64 a) { return make_df(-a.hi, -a.lo); }
__device__ __forceinline__ df64 sub(df64 a, df64 b) { return add(a, neg(b)); }
__device__ __forceinline__ df64 add(df64 a, float b) {
  df64 s = two_sum(a.hi, b);
  s.lo = __fadd_rn(s.lo, a.lo);
  return quick_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ df64 mul(df64 a, df64 b) {
  df64 p = two_prod(a.hi, b.hi);
  p.lo = __fmaf_rn(a.hi, b.lo, p.lo);
  p.lo = __fmaf_rn(a.lo, b.hi, p.lo);
  return quick_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ df64 mul(df64 a, float b) {
  df64 p = two_prod(a.hi, b);
  p.lo = __fmaf_rn(a.lo, b, p.lo);
  return quick_two_sum(p.hi, p.lo);
}
// a*b + c: the product's exact high part (FMA two-product) and its cross terms go into one
// sloppy double-float addition with c, without normalising the product first (14 FP32 ops
// instead of 17; error bound of the same shape, ~2^-47 (|a b| + |c|)).
__device__ __forceinline__ df64 fma_(df64 a, df64 b, df64 c) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  df64 s = two_sum(c.hi, p);
  s.lo = __fadd_rn(s.lo, __fadd_rn(c.lo, e));
  return quick_two_sum(s.hi, s.lo);
}
// 2^e as a float for e in [-126, 127] (built from the exponent field: no conversion unit)
__device__ __forceinline__ float pow2f(int e) { return __int_as_float((e + 127) << 23); }
// a * 2^e, exact while the results stay normal: one multiply for |e| <= 126 (constant e folds
// to it), two for |e| <= 252 (the range exp_tab needs)
__device__ __forceinline__ float scale2f(float a, int e) {
  if (e >= -126 && e <= 127) return a * pow2f(e);
  const int e1 = e >> 1;
  return a * pow2f(e1) * pow2f(e - e1);
}
__device__ __forceinline__ df64 scale2(df64 a, int e) { return make_df(scale2f(a.hi, e), scale2f(a.lo, e)); }

__device__ __forceinline__ df64 div(df64 a, df64 b) {
  float q1 = __fdiv_rn(a.hi, b.hi);
  df64 r = sub(a, mul(b, q1));
  float q2 = __fdiv_rn(r.hi, b.hi);
  r = sub(r, mul(b, q2));
  float q3 = __fdiv_rn(r.hi, b.hi);
  df64 q = quick_two_sum(q1, q2);
  return add(q, q3);
}
__device__ __forceinline__ df64 recip(df64 b) { return div(make_df(1.f), b); }

// sqrt by one Newton correction of the float root: s + (a - s^2) / (2 s)
__device__ __forceinline__ df64 sqrt_(df64 a) {
  if (a.hi <= 0.f) return make_df(0.f);
  float s = sqrtf(a.hi);
  df64 r = sub(a, two_prod(s, s));
  float c = __fdiv_rn(r.hi, 2.f * s);
  return quick_two_sum(s, c);
}

// 1/sqrt(a), a > 0: the float estimate y corrected by the binomial series of (1 - h)^(-1/2),
//   1/sqrt(a) = y (1 + h/2 + 3 h^2/8 + ...),  h = 1 - a y^2,
// where a y^2 is formed in double-float, h = hh + hl is kept as an unevaluated pair (1 - t.hi
// is exact, |h| ~ 2^-22) and the leading correction y hh is an exact product, so that only
// terms below 2^-46 y are rounded in single precision.  The omitted 5 h^3/16 is ~2^-64.
// Measured on a CPU emulation of these operations (20000 inputs over e^[-10,10], estimates
// perturbed by up to 2 ulp): relative error <= 2^-47.1, mean 2^-50.
__device__ __forceinline__ df64 rsqrt_(df64 a) {
  const float y = rsqrtf(a.hi);
  const df64 t = mul(a, two_prod(y, y));
  const float hh = __fsub_rn(1.f, t.hi), hl = -t.lo;
  const float h = __fadd_rn(hh, hl);
  const df64 c = two_prod(y, hh);
  float rest = __fmaf_rn(y, hl, c.lo);
  rest = __fmaf_rn(__fmul_rn(__fmul_rn(y, h), h), 0.75f, rest);   // y (hl + 3/4 h^2) + the product's tail
  df64 r = quick_two_sum(y, __fmul_rn(c.hi, 0.5f));
  r.lo = __fmaf_rn(rest, 0.5f, r.lo);
  return quick_two_sum(r.hi, r.lo);
}

// ---- exp: table-driven reduction x = k ln2/256 + r, |r| <= ln2/512 ----
// Table T[j] = 2^(j/256) stored as df64 (exp2_table.cuh); copied into shared memory
// once per CTA by load_exp_table().
#define GPK_EXP_TABLE 256
#include "exp2_table.cuh"

// ln2/256 = 0.0027076061740622863 as a df64 (hi + lo exact to 3.4e-19)
__device__ __forceinline__ df64 ln2_over_256() { return make_df(2.707606182e-03f, -7.440055516e-12f); }

// NARROW: the domain [-87, 88]; below it the result (< 1.6e-38, already subnormal in its high
// word) is flushed to zero, so that the final scaling 2^m has m in [-126, 126] and takes one
// multiply per word instead of the two-step range-checked one
template <bool NARROW = false, typename Tab>
__device__ __forceinline__ df64 exp_tab(df64 x, const Tab& tab) {
  if (x.hi < (NARROW ? -87.0f : -103.0f)) return make_df(0.f);
  if (x.hi > 88.0f) return make_df(__int_as_float(0x7f800000), 0.f);
  const float inv = 369.32993f;  // 256 / ln 2
  // k = round(x / (ln2/256)) by the 1.5*2^23 magic addition (|x * inv| < 2^22 here): the
  // rounding and the integer both come from one FP32 add, with no conversion instruction
  const float kb = __fadd_rn(x.hi * inv, 12582912.f);
  const float kf = __fsub_rn(kb, 12582912.f);
  const int k = __float_as_int(kb) - 0x4B400000;
  df64 r = sub(x, mul(ln2_over_256(), kf));
  // exp(r) - 1 = r + r^2/2 + r^3/6 + r^4/24  (|r| < 1.4e-3; next term < 4e-17)
  df64 r2 = mul(r, r);
  float t = r.hi * r2.hi * (0.16666667f + r.hi * 0.041666668f);
  df64 p = add(add(r, scale2(r2, -1)), t);
  df64 e = add(p, 1.0f);
  int j = k & (GPK_EXP_TABLE - 1);
  int m = k >> 8;  // arithmetic shift: floor(k / 256)
  float2 tj = tab[j];
  df64 res = mul(make_df(tj.x, tj.y), e);
  if (NARROW) {
    const float s2m = pow2f(m);
    return make_df(res.hi * s2m, res.lo * s2m);
  }
  return scale2(res, m);
}

// log by one Newton step on exp: y1 = y0 + x exp(-y0) - 1
template <typename Tab>
__device__ __forceinline__ df64 log_tab(df64 x, const Tab& tab) {
  float y0 = logf(x.hi);
  df64 ey = exp_tab(make_df(-y0), tab);
  df64 c = sub(mul(x, ey), make_df(1.f));
  return add(make_df(y0), c);
}

// ---- warp reductions ----
__device__ __forceinline__ df64 shfl_xor(df64 a, int m) {
  return make_df(__shfl_xor_sync(0xffffffffu, a.hi, m), __shfl_xor_sync(0xffffffffu, a.lo, m));
}
__device__ __forceinline__ float shfl_xor(float a, int m) { return __shfl_xor_sync(0xffffffffu, a, m); }
__device__ __forceinline__ df64 shfl_idx(df64 a, int src) {
  return make_df(__shfl_sync(0xffffffffu, a.hi, src), __shfl_sync(0xffffffffu, a.lo, src));
}
__device__ __forceinline__ float shfl_idx(float a, int src) { return __shfl_sync(0xffffffffu, a, src); }
__device__ __forceinline__ df64 warp_sum(df64 a) {
#pragma unroll
  for (int m = 16; m > 0; m >>= 1) a = add(a, shfl_xor(a, m));
  return a;
}
__device__ __forceinline__ float warp_sum(float a) {
#pragma unroll
  for (int m = 16; m > 0; m >>= 1) a += __shfl_xor_sync(0xffffffffu, a, m);
  return a;
}
// ---- float overloads so templated kernels compile for T = float ----
__device__ __forceinline__ float add(float a, float b) { return a + b; }
__device__ __forceinline__ float sub(float a, float b) { return a - b; }
__device__ __forceinline__ float mul(float a, float b) { return a * b; }
__device__ __forceinline__ float neg(float a) { return -a; }
__device__ __forceinline__ float fma_(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float recip(float b) { return __fdiv_rn(1.f, b); }
__device__ __forceinline__ float sqrt_(float a) { return sqrtf(fmaxf(a, 0.f)); }
__device__ __forceinline__ float rsqrt_(float a) { return __frsqrt_rn(a); }
__device__ __forceinline__ float scale2(float a, int e) { return scale2f(a, e); }
template <typename Tab> __device__ __forceinline__ float exp_tab(float x, const Tab&) { return expf(x); }
template <typename Tab> __device__ __forceinline__ float log_tab(float x, const Tab&) { return logf(x); }
// The exp of the psi2 pair sweeps (one per pair and point, the bulk of those kernels): the
// double-float exp_tab, or in FP32 CUDA's __expf intrinsic (documented maximum error
// 2 + floor(|1.173 x|) ulp; the terms that dominate a sweep's sums have |x| near 0, and the
// FP32 path's statistics are held to 1e-5 and its gradients to 1e-4 relative).
template <typename Tab> __device__ __forceinline__ df64 exp_pair(df64 x, const Tab& tab) { return exp_tab<true>(x, tab); }
template <typename Tab> __device__ __forceinline__ float exp_pair(float x, const Tab&) { return __expf(x); }

// Warp sums of K values at once (K a power of two <= 32): in each of the first log2 K steps
// of the butterfly a lane keeps half of its values and adds its partner's copies of them,
// trading the other half, so the K sums take K - 1 + 5 - log2 K exchanges instead of 5 K.
// On return v[0] of lane l holds the warp total of value l >> (5 - log2 K).
template <int K, typename T>
__device__ __forceinline__ void warp_sum_many(T (&v)[K]) {
  static_assert(K >= 1 && K <= 32 && (K & (K - 1)) == 0, "K must be a power of two <= 32");
  const int lane = threadIdx.x & 31;
  int off = 16;
#pragma unroll
  for (int n = K; n > 1; n >>= 1, off >>= 1) {
    const bool up = (lane & off) != 0;   // this lane keeps the upper half of the n values
#pragma unroll
    for (int i = 0; i < n / 2; ++i) {
      const T keep = up ? v[i + n / 2] : v[i];
      const T send = up ? v[i] : v[i + n / 2];
      v[i] = add(keep, shfl_xor(send, off));
    }
  }
#pragma unroll
  for (; off > 0; off >>= 1) v[0] = add(v[0], shfl_xor(v[0], off));
}

// conversions between storage (double / float) and compute (df64 / float) types
// A compute-type element read as one 8-byte access (df64) when its address is known to be
// 8-byte aligned (df64 itself is only 4-byte aligned, so plain loads may split in two).
__device__ __forceinline__ df64 ld_al8(const df64* p) {
  const float2 v = *reinterpret_cast<const float2*>(p);
  return make_df(v.x, v.y);
}
__device__ __forceinline__ float ld_al8(const float* p) { return *p; }

template <typename T> struct Num;
template <> struct Num<df64> {
  typedef double store_t;
  __device__ static __forceinline__ df64 ld(double x) { return df_from_double(x); }
  __device__ static __forceinline__ double st(df64 x) { return df_to_double(x); }
  __device__ static __forceinline__ df64 c(float x) { return make_df(x); }
  __device__ static __forceinline__ df64 zero() { return make_df(0.f); }
  __device__ static __forceinline__ float approx(df64 x) { return x.hi; }
};
template <> struct Num<float> {
  typedef float store_t;
  __device__ static __forceinline__ float ld(float x) { return x; }
  __device__ static __forceinline__ float st(float x) { return x; }
  __device__ static __forceinline__ float c(float x) { return x; }
  __device__ static __forceinline__ float zero() { return 0.f; }
  __device__ static __forceinline__ float approx(float x) { return x; }
};

// the exp table lives in shared memory; every kernel that calls exp_tab loads it first
__device__ __forceinline__ void load_exp_table(float2* s_tab) {
  for (int i = threadIdx.x; i < GPK_EXP_TABLE; i += blockDim.x) s_tab[i] = kExp2Tab[i];
}
