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

}  // namespace qbg
