// lbm_df64.cuh -- float-float ("double-float") arithmetic on the FP32 pipes.
//
// GB300 executes FP64 at 1/64 of its FP32 rate, which makes an FP64 collide-stream step
// compute-bound far below the HBM roof.  A value v is kept as an unevaluated sum hi + lo of
// two floats with |lo| <= ulp(hi)/2, i.e. a 48-bit significand.  The populations are stored
// as their deviation from the weights, g = f - w (|g| << |f|), so the absolute precision of
// f is |g| * 2^-48, at or below the FP64 rounding of f itself.
//
// The algorithms are the classical error-free transformations:
//   two_sum (Knuth, 1969), fast_two_sum (Dekker, 1971), two_prod with a fused multiply-add;
//   addition and multiplication in the "sloppy" forms of the double-double / double-float
//   libraries (Hida, Li and Bailey, QD, 2001; Thall, "Extended-precision floating-point
//   numbers for GPU computation", 2006); the reciprocal by one Newton step in float-float.
// All operations use explicitly rounded FP32 intrinsics so the compiler cannot reassociate
// or contract them.
#pragma once

#include <cuda_runtime.h>

namespace lbm {

struct dd {
  float hi, lo;

  __host__ __device__ __forceinline__ dd() : hi(0.f), lo(0.f) {}
  __host__ __device__ __forceinline__ dd(float h, float l) : hi(h), lo(l) {}
  __host__ __device__ __forceinline__ dd(int i) : hi((float)i), lo(0.f) {}
  __host__ __device__ __forceinline__ dd(float f) : hi(f), lo(0.f) {}
  // split of a double into the nearest float and the float nearest the remainder
  __host__ __device__ __forceinline__ dd(double d) {
    hi = (float)d;
    lo = (float)(d - (double)hi);
  }
  __host__ __device__ __forceinline__ explicit operator double() const { return (double)hi + (double)lo; }
};

#ifdef __CUDACC__
__device__ __forceinline__ dd two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return dd(s, e);
}

__device__ __forceinline__ dd fast_two_sum(float a, float b) {  // requires |a| >= |b| (or a == 0)
  const float s = __fadd_rn(a, b);
  const float e = __fsub_rn(b, __fsub_rn(s, a));
  return dd(s, e);
}

__device__ __forceinline__ dd operator+(dd a, dd b) {
  dd s = two_sum(a.hi, b.hi);
  const float e = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
  return fast_two_sum(s.hi, e);
}

// a + b without the closing renormalisation, for sums that feed further sums or products: the
// leading parts are added exactly (two_sum) and every rounding error is kept in the trailing
// part, so a chain of such additions is the cascaded summation of Ogita, Rump and Oishi
// ("Accurate sum and dot product", 2005), renormalised by the first full addition after it.
__device__ __forceinline__ dd add_lazy(dd a, dd b) {
  const dd s = two_sum(a.hi, b.hi);
  return dd(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}

__device__ __forceinline__ dd operator-(dd a) { return dd(-a.hi, -a.lo); }

__device__ __forceinline__ dd operator-(dd a, dd b) { return a + (-b); }

// The product is left as the pair (p, e) with p = fl(a.hi b.hi) and e the rounding error of
// p plus the cross terms, |e| <= ~2^-22 |p|, without the closing fast_two_sum: every consumer
// (two_sum-based addition, another product, the reciprocal, a store) is exact or error-free
// in its leading part for such a pair, and the renormalisation happens in the next addition.
__device__ __forceinline__ dd operator*(dd a, dd b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return dd(p, e);
}

// 1 / b: float reciprocal refined by one Newton step r + r (1 - b r) in float-float
__device__ __forceinline__ dd recip(dd b) {
  const float r = __frcp_rn(b.hi);
  const dd br = b * dd(r, 0.f);
  const float e = __fsub_rn(__fsub_rn(1.0f, br.hi), br.lo);
  return fast_two_sum(r, __fmul_rn(r, e));
}

__device__ __forceinline__ dd operator/(dd a, dd b) { return a * recip(b); }

__device__ __forceinline__ bool operator!=(dd a, dd b) { return a.hi != b.hi || a.lo != b.lo; }

__device__ __forceinline__ dd& operator+=(dd& a, dd b) { return a = a + b; }
__device__ __forceinline__ dd& operator-=(dd& a, dd b) { return a = a - b; }
__device__ __forceinline__ dd& operator*=(dd& a, dd b) { return a = a * b; }
#endif

}  // namespace lbm
