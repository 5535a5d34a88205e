// lbm_pf2.cuh -- two FP32 values in one 64-bit register pair, added, multiplied and fused
// multiply-added by one packed instruction (PTX add / sub / mul / fma .rn.f32x2, sm_100 and
// later).  Kernels that advance two nodes per thread carry every FP32 quantity of the
// collision as a pf2 (lane 0: first node, lane 1: second node), so the arithmetic of both
// nodes issues once.  Each lane is rounded exactly as the scalar FP32 operation, except that the
// code generator may merge a product with an addition that consumes it (see pmul_exact): code
// whose rounding must match the scalar code writes its multiply-adds as explicit FMAs.
#pragma once

#include <cuda_fp16.h>

#include "lbm_df64.cuh"

namespace lbm {

struct pf2 {
  unsigned long long r;
  pf2() = default;
  __device__ __forceinline__ pf2(float a) { asm("mov.b64 %0, {%1, %1};" : "=l"(r) : "f"(a)); }
  __device__ __forceinline__ pf2(float a, float b) { asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b)); }
  __device__ __forceinline__ float lo() const {
    float a;
    asm("{.reg .f32 t; mov.b64 {%0, t}, %1;}" : "=f"(a) : "l"(r));
    return a;
  }
  __device__ __forceinline__ float hi() const {
    float b;
    asm("{.reg .f32 t; mov.b64 {t, %0}, %1;}" : "=f"(b) : "l"(r));
    return b;
  }
};

__device__ __forceinline__ pf2 operator+(pf2 a, pf2 b) {
  pf2 o;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(o.r) : "l"(a.r), "l"(b.r));
  return o;
}
__device__ __forceinline__ pf2 operator-(pf2 a, pf2 b) {
  pf2 o;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(o.r) : "l"(a.r), "l"(b.r));
  return o;
}
__device__ __forceinline__ pf2 operator*(pf2 a, pf2 b) {
  pf2 o;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(o.r) : "l"(a.r), "l"(b.r));
  return o;
}
__device__ __forceinline__ pf2 operator-(pf2 a) {  // flips both sign bits
  pf2 o;
  o.r = a.r ^ 0x8000000080000000ull;
  return o;
}
__device__ __forceinline__ pf2& operator+=(pf2& a, pf2 b) { return a = a + b; }
__device__ __forceinline__ pf2 pfma(pf2 a, pf2 b, pf2 c) {
  pf2 o;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(o.r) : "l"(a.r), "l"(b.r), "l"(c.r));
  return o;
}

// The multiply-add shapes of the collision, fused for pf2 (the scalar forms are in
// lbm_common.cuh): c + a b, c - a b, a b + c, a b - c, and a b + c of a stored value.
__device__ __forceinline__ pf2 add_prod(pf2 c, pf2 a, pf2 b) { return pfma(a, b, c); }
__device__ __forceinline__ pf2 sub_prod(pf2 c, pf2 a, pf2 b) { return pfma(-a, b, c); }
__device__ __forceinline__ pf2 prod_add(pf2 a, pf2 b, pf2 c) { return pfma(a, b, c); }
__device__ __forceinline__ pf2 prod_sub(pf2 a, pf2 b, pf2 c) { return pfma(a, b, -c); }
__device__ __forceinline__ pf2 prod_add_out(pf2 a, pf2 b, pf2 c) { return pfma(a, b, c); }

__device__ __forceinline__ pf2 pair_recip(pf2 r) { return pf2(__frcp_rn(r.lo()), __frcp_rn(r.hi())); }
__device__ __forceinline__ bool nonzero_bits(pf2 v) { return v.r != 0ull; }

// -0 in both lanes, read from constant memory so that the code generator cannot see the addend.
// The code generator merges a packed multiply with a packed addition that consumes the product
// into one packed FMA even when both carry an explicit rounding mode (and it treats an FMA with a
// literal -0 addend as a multiply), which would change the rounding of the error-free
// transformations below.  A product formed as fma(a, b, kNegZero2) equals the rounded product
// (x + (-0) = x for every x, signed zeros included) and is never merged.
static __constant__ unsigned long long kNegZero2 = 0x8000000080000000ull;
__device__ __forceinline__ pf2 pmul_exact(pf2 a, pf2 b) {
  pf2 o;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(o.r) : "l"(a.r), "l"(b.r), "l"(kNegZero2));
  return o;
}

// Float-float values of two nodes: the operations of lbm_df64.cuh on packed pairs, step by step
// the same roundings, so each lane equals the dd result of its node bitwise.
struct pdd {
  pf2 hi, lo;
  pdd() = default;
  __device__ __forceinline__ pdd(pf2 h, pf2 l) : hi(h), lo(l) {}
  __device__ __forceinline__ pdd(int i) : hi((float)i), lo(0.f) {}
  __device__ __forceinline__ pdd(float f) : hi(f), lo(0.f) {}
  __device__ __forceinline__ pdd(double d) {
    const dd t(d);
    hi = pf2(t.hi);
    lo = pf2(t.lo);
  }
  __device__ __forceinline__ pdd(dd d) : hi(d.hi), lo(d.lo) {}  // the same value in both lanes
};

__device__ __forceinline__ pdd two_sum(pf2 a, pf2 b) {
  const pf2 s = a + b;
  const pf2 bb = s - a;
  return pdd(s, (a - (s - bb)) + (b - bb));
}
// two_sum(a, -b) without the negations: (-b) - bb = -(b + bb) exactly
__device__ __forceinline__ pdd two_diff(pf2 a, pf2 b) {
  const pf2 s = a - b;
  const pf2 bb = s - a;
  return pdd(s, (a - (s - bb)) - (b + bb));
}
__device__ __forceinline__ pdd fast_two_sum(pf2 a, pf2 b) {
  const pf2 s = a + b;
  return pdd(s, b - (s - a));
}
__device__ __forceinline__ pdd operator+(pdd a, pdd b) {
  const pdd s = two_sum(a.hi, b.hi);
  return fast_two_sum(s.hi, s.lo + (a.lo + b.lo));
}
__device__ __forceinline__ pdd operator-(pdd a, pdd b) {
  const pdd s = two_diff(a.hi, b.hi);
  return fast_two_sum(s.hi, s.lo + (a.lo - b.lo));
}
__device__ __forceinline__ pdd operator-(pdd a) { return pdd(-a.hi, -a.lo); }
__device__ __forceinline__ pdd add_lazy(pdd a, pdd b) {
  const pdd s = two_sum(a.hi, b.hi);
  return pdd(s.hi, s.lo + (a.lo + b.lo));
}
__device__ __forceinline__ pdd sub_lazy(pdd a, pdd b) {
  const pdd s = two_diff(a.hi, b.hi);
  return pdd(s.hi, s.lo + (a.lo - b.lo));
}
__device__ __forceinline__ pdd operator*(pdd a, pdd b) {
  const pf2 p = pmul_exact(a.hi, b.hi);
  pf2 e = pfma(a.hi, b.hi, -p);
  e = pfma(a.hi, b.lo, e);
  e = pfma(a.lo, b.hi, e);
  return pdd(p, e);
}
__device__ __forceinline__ pdd recip(pdd b) {
  const pf2 r(__frcp_rn(b.hi.lo()), __frcp_rn(b.hi.hi()));
  const pdd br = b * pdd(r, pf2(0.f));
  const pf2 e = (pf2(1.0f) - br.hi) - br.lo;
  return fast_two_sum(r, pmul_exact(r, e));
}
__device__ __forceinline__ pdd ladd(pdd a, pdd b) { return add_lazy(a, b); }
__device__ __forceinline__ pdd lsub(pdd a, pdd b) { return sub_lazy(a, b); }
// the multiply-add shapes as for dd (lbm_common.cuh), taking float-float parameters in either place
__device__ __forceinline__ pdd add_prod(pdd c, pdd a, pdd b) { return add_lazy(c, a * b); }
__device__ __forceinline__ pdd sub_prod(pdd c, pdd a, pdd b) { return sub_lazy(c, a * b); }
__device__ __forceinline__ pdd prod_add(pdd a, pdd b, pdd c) { return add_lazy(a * b, c); }
__device__ __forceinline__ pdd prod_sub(pdd a, pdd b, pdd c) { return sub_lazy(a * b, c); }
__device__ __forceinline__ pdd prod_add_out(pdd a, pdd b, pdd c) { return a * b + c; }
__device__ __forceinline__ pdd pair_recip(pdd r) { return recip(r); }
__device__ __forceinline__ bool nonzero_bits(pdd v) { return v.hi.r != 0ull || v.lo.r != 0ull; }

// two nodes' values as one packed value
__device__ __forceinline__ pf2 pack2(float a, float b) { return pf2(a, b); }
__device__ __forceinline__ pdd pack2(dd a, dd b) { return pdd(pf2(a.hi, b.hi), pf2(a.lo, b.lo)); }
template <class C>
struct Packed;
template <>
struct Packed<float> {
  using type = pf2;
};
template <>
struct Packed<dd> {
  using type = pdd;
};

}  // namespace lbm
