// qbg_df32.cuh -- double-float arithmetic: a value is the unevaluated sum
// hi + lo of two FP32 numbers (|lo| <= ulp(hi)/2), carrying ~48 significant
// bits.  GB300 executes FP32 at 72x its FP64 rate, so transforms written in
// this type reach FP64-class accuracy for this path (~1e-14 relative,
// norm-wise) several times faster than native FP64.
//
// Algorithms (published): addition uses Knuth's TwoSum on the high parts
// followed by a fast renormalisation (the "sloppy" double-float sum of
// Dekker, 1971, and Hida-Li-Bailey's QD library); multiplication uses the
// FMA form of Dekker's TwoProduct.  The sloppy sum's error is bounded by a
// few 2^-48 of |a| + |b|, which is what a norm-stable FFT needs.
#pragma once
#include <cuda_runtime.h>

namespace qbg {

struct df32 {
  float hi, lo;
  df32() = default;
  __host__ __device__ __forceinline__ constexpr df32(float h, float l) : hi(h), lo(l) {}
  __host__ __device__ __forceinline__ df32(double d)
      : hi((float)d), lo((float)(d - (double)(float)d)) {}
  __host__ __device__ __forceinline__ df32(int i) : hi((float)i), lo(0.f) {}
  __host__ __device__ __forceinline__ explicit operator double() const {
    return (double)hi + (double)lo;
  }
};

__device__ __forceinline__ df32 df_renorm(float s, float e) {
  const float h = s + e;
  return df32(h, e - (h - s));
}

// Sum without the final renormalisation: (s, e) with s = fl(a.hi + b.hi),
// e = exact error of that sum + a.lo + b.lo.  The pair may carry |e| of a
// few ulp(s) (more after cancellation), but its absolute error stays a few
// 2^-47 of the operands' magnitude, which is the norm-wise accuracy an FFT
// needs; every consumer (sum, product, conversion) accepts such pairs.
__device__ __forceinline__ df32 operator+(df32 a, df32 b) {
  const float s = a.hi + b.hi;
  const float bb = s - a.hi;
  float e = (a.hi - (s - bb)) + (b.hi - bb);
  e += a.lo + b.lo;
  return df32(s, e);
}
// exact scaling by a power of two
__host__ __device__ __forceinline__ df32 df_scale2(df32 a, float p2) { return df32(a.hi * p2, a.lo * p2); }
__device__ __forceinline__ df32 operator-(df32 a) { return df32(-a.hi, -a.lo); }
__device__ __forceinline__ df32 operator-(df32 a, df32 b) { return a + (-b); }
// The FMA-exact error of hi*hi plus the two cross terms stays below half an
// ulp of the product (for normalised inputs), so the pair (p, e) is already
// normalised to within a rounding and needs no extra renormalisation.
__device__ __forceinline__ df32 operator*(df32 a, df32 b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return df32(p, e);
}
__device__ __forceinline__ df32& operator+=(df32& a, df32 b) { return a = a + b; }
__device__ __forceinline__ df32& operator*=(df32& a, df32 b) { return a = a * b; }

struct __align__(16) df32c {
  df32 x, y;
};

// FP64 -> double-float from the bit pattern, with no FP64 instruction (GB300
// runs FP64 at 1/72 of the FP32 rate, conversions included): hi takes the
// 24 leading significand bits (truncated), lo the next 23 as an exact
// integer times a power of two, so hi + lo carries 47 bits of x.  |x| below
// 2^-80 (lo) or 2^-126 (hi) flushes to zero: the path's values are
// normalised to order one.
__device__ __forceinline__ df32 df32_from_f64(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
  const int E = (int)((b >> 52) & 0x7FF);
  const int fe = E - 1023 + 127;
  if (fe <= 0) return df32(0.f, 0.f);
  const float hi = __uint_as_float(sign | ((unsigned)fe << 23) | (unsigned)((b >> 29) & 0x7FFFFF));
  const int le = E - 1069 + 127;  // exponent of the lo part's unit
  float lo = 0.f;
  if (le > 0) {
    const unsigned r = (unsigned)(b & 0x1FFFFFFFu) >> 6;  // 23 bits
    const float mag = __uint_as_float(0x4B000000u | r) - 8388608.0f;  // exact integer r
    lo = __uint_as_float(sign | __float_as_uint(mag * __uint_as_float((unsigned)le << 23)));
  }
  return df32(hi, lo);
}
// FP64 -> FP32 rounded to nearest (ties away from zero) from the bit
// pattern: half a unit of the 24-bit significand is added to the magnitude
// bits before truncation (a carry into the exponent is the correct
// rounding), so no FP64 instruction is issued.  |x| below 2^-126 gives zero.
__device__ __forceinline__ float f32_from_f64_rn(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned long long m = (b & 0x7FFFFFFFFFFFFFFFull) + (1ull << 28);
  const int fe = (int)(m >> 52) - 1023 + 127;
  if (fe <= 0) return 0.f;
  return __uint_as_float(((unsigned)(b >> 32) & 0x80000000u) | ((unsigned)fe << 23) |
                         (unsigned)((m >> 29) & 0x7FFFFF));
}
// FP32 -> FP64 from the bit pattern (exact for normal numbers; zero and
// subnormal inputs give zero), no FP64 instruction
__device__ __forceinline__ double f64_from_f32(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xFF;
  if (e == 0) return 0.0;
  const unsigned long long b = ((unsigned long long)(u & 0x80000000u) << 32) |
                               ((unsigned long long)(e - 127 + 1023) << 52) |
                               ((unsigned long long)(u & 0x7FFFFFu) << 29);
  return __longlong_as_double((long long)b);
}
// double-float -> FP64: one FP64 add
__device__ __forceinline__ double f64_from_df32(df32 a) {
  return f64_from_f32(a.hi) + f64_from_f32(a.lo);
}

}  // namespace qbg
