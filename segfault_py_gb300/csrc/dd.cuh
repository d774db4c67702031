// dd.cuh -- double-float ("dd") arithmetic on the FP32 pipe.
//
// A value is the unevaluated sum hi + lo of two floats with |lo| <= ulp(hi)/2,
// about 48 significant bits.  GB300's FP64 pipe runs at 1/64 of the FP32 rate
// and one warp's FP64 instruction occupies its sub-partition's FP64 unit for
// 64 cycles, so a quartet evaluated with dd operations (7 to 15 FP32
// instructions each) is several times faster than the same quartet in FP64,
// with a relative rounding error near 2^-44 instead of 2^-53.
//
// The building blocks are the error-free transformations of Knuth (TwoSum),
// Dekker (FastTwoSum) and the FMA form of TwoProduct; the "sloppy" addition
// and the multiplication follow the double-double algorithms of Hida, Li and
// Bailey (QD library paper, 2001), written here for float pairs.
#pragma once
#include <cuda_runtime.h>

namespace sf {

struct dd {
  float hi, lo;
  dd() = default;
  __host__ __device__ constexpr dd(float h, float l) : hi(h), lo(l) {}
  __host__ __device__ constexpr dd(float h) : hi(h), lo(0.0f) {}
  __host__ __device__ constexpr dd(int i) : hi((float)i), lo(0.0f) {}
  // split of a double (constant-folded for compile-time constants)
  __host__ __device__ constexpr explicit dd(double d) : hi((float)d), lo((float)(d - (double)(float)d)) {}
};

__device__ __forceinline__ dd dd_fast_two_sum(float a, float b) {   // |a| >= |b|
  const float s = a + b;
  return dd(s, b - (s - a));
}

__device__ __forceinline__ dd dd_two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  return dd(s, (a - (s - bb)) + (b - bb));
}

__device__ __forceinline__ dd operator+(dd a, dd b) {
  dd s = dd_two_sum(a.hi, b.hi);
  return dd_fast_two_sum(s.hi, s.lo + (a.lo + b.lo));
}
__device__ __forceinline__ dd operator-(dd a) { return dd(-a.hi, -a.lo); }
__device__ __forceinline__ dd operator-(dd a, dd b) { return a + (-b); }

__device__ __forceinline__ dd operator*(dd a, dd b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  return dd_fast_two_sum(p, e);
}
__device__ __forceinline__ dd operator*(dd a, float b) {
  const float p = a.hi * b;
  float e = fmaf(a.hi, b, -p);
  e = fmaf(a.lo, b, e);
  return dd_fast_two_sum(p, e);
}
__device__ __forceinline__ dd operator*(float b, dd a) { return a * b; }
__device__ __forceinline__ dd operator*(dd a, int b) { return a * (float)b; }
__device__ __forceinline__ dd operator*(int b, dd a) { return a * (float)b; }

// a*b + c with one renormalisation
__device__ __forceinline__ dd dd_fma(dd a, dd b, dd c) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  dd s = dd_two_sum(p, c.hi);
  return dd_fast_two_sum(s.hi, s.lo + (e + c.lo));
}

__device__ __forceinline__ dd &operator+=(dd &a, dd b) { return a = a + b; }
__device__ __forceinline__ dd &operator-=(dd &a, dd b) { return a = a - b; }
__device__ __forceinline__ dd &operator*=(dd &a, dd b) { return a = a * b; }
__device__ __forceinline__ dd &operator*=(dd &a, float b) { return a = a * b; }

__device__ __forceinline__ bool operator>=(dd a, float b) { return a.hi > b || (a.hi == b && a.lo >= 0.0f); }

// 1/a: FP32 reciprocal seed, one Newton step y + y (1 - a y) in dd
__device__ __forceinline__ dd dd_recip(dd a) {
  const float y0 = 1.0f / a.hi;
  const dd y(y0);
  const dd r = dd(1.0f) - a * y;
  return y + y * r;
}

// 1/sqrt(a): FP32 seed, one Newton step y (3/2 - a/2 y^2) in dd
__device__ __forceinline__ dd dd_rsqrt(dd a) {
  const dd y(rsqrtf(a.hi));
  const dd h = a * 0.5f;
  return y * (dd(1.5f) - h * (y * y));
}

__device__ __forceinline__ dd dd_shfl_xor(unsigned mask, dd v, int lane_mask) {
  return dd(__shfl_xor_sync(mask, v.hi, lane_mask), __shfl_xor_sync(mask, v.lo, lane_mask));
}

__device__ __forceinline__ dd dd_ldg(const dd *p) {
  const float2 v = __ldg(reinterpret_cast<const float2 *>(p));
  return dd(v.x, v.y);
}

}  // namespace sf
