// dfloat.cuh -- float-float ("double-word") numbers for the FP64-accurate
// parts of the MIXED Poisson solve on GB300.
//
// GB300 executes FP64 at 1/64 of its FP32 rate, so a 3D FFT in FP64 is bound
// by the FP64 pipe. A value held as an unevaluated sum hi + lo of two floats
// (|lo| <= ulp(hi)/2) carries 48 significand bits; its arithmetic runs on
// the FP32 pipes with error-free transformations:
//   two_sum      Knuth's TwoSum: s = RN(a + b) and the exact error a + b - s
//   fast_two_sum Dekker's Fast2Sum (|a| >= |b| or a = 0)
//   product      RN(a b) and its exact error fma(a, b, -RN(a b))
// Addition is the "sloppy" double-word sum (Dekker 1971; analysed by Joldes,
// Muller and Popescu, ACM TOMS 44(2), 2017): TwoSum of the high words, the
// low words added to its error, Fast2Sum to renormalise. Its error is bounded
// relative to |a| + |b| (not to |a + b|), which is the bound FFT error
// analysis uses. Multiplication is the FMA double-word product: the exact
// product of the high words plus the two cross terms, renormalised. All steps
// use the _rn intrinsics so that the compiler never contracts them into other
// operations.
//
// Range: the exponent range is FP32's. The fields of the Poisson solve lie
// many decades inside it; values below FLT_MIN lose their low word.
#pragma once
#include <cuda_runtime.h>

namespace icep {

struct dfl {
  float hi, lo;
  dfl() = default;
  __host__ __device__ constexpr dfl(int v) : hi((float)v), lo(0.f) {}
  __host__ __device__ constexpr dfl(float v) : hi(v), lo(0.f) {}
  __host__ __device__ constexpr dfl(float h, float l) : hi(h), lo(l) {}
  // Nearest float plus the rounded remainder. Host-side (tables and scalar
  // kernel arguments); device code builds dfl values from floats only.
  __host__ static dfl from_double(double v) {
    const float h = (float)v;
    return dfl(h, (float)(v - (double)h));
  }
  __host__ __device__ double to_double() const { return (double)hi + (double)lo; }
};

#ifdef __CUDACC__
__device__ __forceinline__ dfl two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return dfl(s, e);
}
__device__ __forceinline__ dfl fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return dfl(s, __fsub_rn(b, __fsub_rn(s, a)));
}
__device__ __forceinline__ dfl operator+(dfl a, dfl b) {
  const dfl s = two_sum(a.hi, b.hi);
  return fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ dfl operator-(dfl a) { return dfl(-a.hi, -a.lo); }
__device__ __forceinline__ dfl operator-(dfl a, dfl b) { return a + (-b); }
__device__ __forceinline__ dfl operator*(dfl a, dfl b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return fast_two_sum(p, e);
}
__device__ __forceinline__ dfl operator*(dfl a, float b) {
  const float p = __fmul_rn(a.hi, b);
  float e = __fmaf_rn(a.hi, b, -p);
  e = __fmaf_rn(a.lo, b, e);
  return fast_two_sum(p, e);
}
__device__ __forceinline__ dfl &operator+=(dfl &a, dfl b) { return a = a + b; }
__device__ __forceinline__ dfl &operator-=(dfl &a, dfl b) { return a = a - b; }
__device__ __forceinline__ dfl &operator*=(dfl &a, dfl b) { return a = a * b; }
// exact product of two floats as a dfl
__device__ __forceinline__ dfl two_prod(float a, float b) {
  const float p = __fmul_rn(a, b);
  return dfl(p, __fmaf_rn(a, b, -p));
}
// the nearest float
__device__ __forceinline__ float to_float(dfl a) { return __fadd_rn(a.hi, a.lo); }
#endif

// x / 2, exactly for the dfl and binary floating-point types
__host__ __device__ __forceinline__ float half_of(float x) { return 0.5f * x; }
__host__ __device__ __forceinline__ double half_of(double x) { return 0.5 * x; }
__host__ __device__ __forceinline__ dfl half_of(dfl x) { return dfl(0.5f * x.hi, 0.5f * x.lo); }

// sqrt(1/2) in each arithmetic type (the radix-8 twiddle)
template <typename R>
__host__ __device__ __forceinline__ R sqrt_half() { return (R)0.70710678118654752440084436210484903928; }
template <>
__host__ __device__ __forceinline__ dfl sqrt_half<dfl>() {
  // hi = RN_32(sqrt(1/2)), lo = RN_32(sqrt(1/2) - hi)
  return dfl(0.707106769084930419921875f, 1.21016174858823433169e-08f);
}

// Conversion of a host double to the arithmetic type R.
template <typename R>
__host__ inline R from_double(double v) { return (R)v; }
template <>
__host__ inline dfl from_double<dfl>(double v) { return dfl::from_double(v); }

}  // namespace icep
