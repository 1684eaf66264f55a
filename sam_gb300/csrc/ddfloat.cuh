// Double-float arithmetic on the FP32 pipe: a value is the unevaluated sum
// hi + lo of two FP32 numbers with |lo| <= ulp(hi) / 2, about 48 significand
// bits.  GB300 issues FP32 at 64 times its FP64 rate, so a transform written
// in these pairs (about ten FP32 operations per FP64 one) runs several times
// faster than in FP64 while keeping FP64-level accuracy for the FFT passes.
//
// Building blocks (error-free transformations, published methods):
//   two_sum      Knuth:   s + e = a + b exactly (6 operations)
//   fast_two_sum Dekker:  s + e = a + b exactly when |a| >= |b| (3)
//   two_prod     FMA:     p + e = a * b exactly (2)
// Addition is the "sloppy" double-float sum (one two_sum on the high parts,
// the low parts added in FP32): its error is below about 3 * 2^-48 (|a| + |b|),
// the norm-wise bound the FFT's error analysis uses (a butterfly's error
// relative to its inputs, not to a cancelled result).  Multiplication keeps
// the three leading partial products; division refines an FP32 quotient once
// with the exact remainder (Dekker).  Every FP32 operation is written with
// the _rn intrinsics so the compiler never contracts a product and a sum into
// one FMA, which would break the error-free transformations.
//
// The exponent range is FP32's: magnitudes below about 1e-38 flush to zero,
// far below the relative accuracy kept (values are O(1) in this code).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace samgpu {

struct dd {
  float hi, lo;
  dd() = default;
  __host__ __device__ constexpr dd(float h, float l) : hi(h), lo(l) {}
  __host__ __device__ constexpr dd(int i) : hi((float)i), lo(0.0f) {}  // exact for |i| < 2^24
  __host__ __device__ constexpr dd(float f) : hi(f), lo(0.0f) {}
  // the nearest pair to a double (53 bits into 48: rounds the low part)
  __host__ __device__ constexpr explicit dd(double x) : hi((float)x), lo((float)(x - (double)(float)x)) {}
  __host__ __device__ explicit operator double() const { return (double)hi + (double)lo; }
};

// complex pair; 16-byte aligned so a value moves as one vector load/store
struct __align__(16) ddc {
  dd x, y;
};

template <typename T> struct IsDD { static constexpr bool value = false; };
template <> struct IsDD<dd> { static constexpr bool value = true; };
template <typename T> inline constexpr bool kIsDD = IsDD<T>::value;

__device__ __forceinline__ dd dd_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return dd(s, e);
}
__device__ __forceinline__ dd dd_fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return dd(s, __fsub_rn(b, __fsub_rn(s, a)));
}

__device__ __forceinline__ dd operator+(dd a, dd b) {
  const dd s = dd_two_sum(a.hi, b.hi);
  return dd_fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ dd operator-(dd a) { return dd(-a.hi, -a.lo); }
__device__ __forceinline__ dd operator-(dd a, dd b) {
  const dd s = dd_two_sum(a.hi, -b.hi);
  return dd_fast_two_sum(s.hi, __fadd_rn(s.lo, __fsub_rn(a.lo, b.lo)));
}
__device__ __forceinline__ dd operator*(dd a, dd b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return dd_fast_two_sum(p, e);
}
// a * b - c * d with one normalisation (the complex products' real parts)
__device__ __forceinline__ dd dd_mul_sub(dd a, dd b, dd c, dd d) {
  const float p1 = __fmul_rn(a.hi, b.hi), p2 = __fmul_rn(c.hi, d.hi);
  float e1 = __fmaf_rn(a.hi, b.hi, -p1), e2 = __fmaf_rn(c.hi, d.hi, -p2);
  const dd s = dd_two_sum(p1, -p2);
  float e = __fadd_rn(s.lo, __fsub_rn(e1, e2));
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  e = __fmaf_rn(-c.hi, d.lo, e);
  e = __fmaf_rn(-c.lo, d.hi, e);
  return dd_fast_two_sum(s.hi, e);
}
// a * b + c * d
__device__ __forceinline__ dd dd_mul_add(dd a, dd b, dd c, dd d) { return dd_mul_sub(a, b, -c, d); }

__device__ __forceinline__ dd operator/(dd a, dd b) {
  const float q1 = __fdiv_rn(a.hi, b.hi);
  const dd r = a - b * dd(q1);
  const float q2 = __fdiv_rn(r.hi, b.hi);
  return dd_fast_two_sum(q1, q2);
}

__device__ __forceinline__ dd& operator+=(dd& a, dd b) { return a = a + b; }
__device__ __forceinline__ dd& operator-=(dd& a, dd b) { return a = a - b; }
__device__ __forceinline__ dd& operator*=(dd& a, dd b) { return a = a * b; }

// comparisons of normalised pairs: the high parts, then the low parts
__device__ __forceinline__ bool operator<(dd a, dd b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ bool operator>(dd a, dd b) { return b < a; }
__device__ __forceinline__ bool operator==(dd a, dd b) { return a.hi == b.hi && a.lo == b.lo; }
__device__ __forceinline__ bool operator!=(dd a, dd b) { return !(a == b); }

__device__ __forceinline__ bool dd_isfinite(dd a) { return isfinite(a.hi) && isfinite(a.lo); }

// Order-preserving 64-bit key of |a| (the high part's magnitude bits, then
// the low part signed to that magnitude, mapped to an increasing unsigned
// code): max |a| over many values is the max of their keys.
__device__ __forceinline__ unsigned long long dd_abs_key(dd a) {
  const bool neg = a.hi < 0.0f || (a.hi == 0.0f && a.lo < 0.0f);
  const float h = neg ? -a.hi : a.hi, l = neg ? -a.lo : a.lo;
  const uint32_t lb = __float_as_uint(l);
  const uint32_t lk = (lb & 0x80000000u) ? ~lb : (lb | 0x80000000u);
  return ((unsigned long long)__float_as_uint(h) << 32) | lk;
}
__host__ __device__ inline double dd_key_value(unsigned long long k) {
  if (k == 0ull) return 0.0;  // no value recorded
  const uint32_t hb = (uint32_t)(k >> 32), lk = (uint32_t)k;
  const uint32_t lb = (lk & 0x80000000u) ? (lk & 0x7FFFFFFFu) : ~lk;
  float h, l;
#ifdef __CUDA_ARCH__
  h = __uint_as_float(hb);
  l = __uint_as_float(lb);
#else
  __builtin_memcpy(&h, &hb, 4);
  __builtin_memcpy(&l, &lb, 4);
#endif
  return (double)h + (double)l;
}

}  // namespace samgpu
