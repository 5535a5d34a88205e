// lbm_pf2.cuh -- two FP32 values in one 64-bit register pair, added, multiplied and fused
// multiply-added by one packed instruction (PTX add / sub / mul / fma .rn.f32x2, sm_100 and
// later).  Kernels that advance two nodes per thread carry every FP32 quantity of the
// collision as a pf2 (lane 0: first node, lane 1: second node), so the arithmetic of both
// nodes issues once.  Each lane is rounded exactly as the scalar FP32 operation.
#pragma once

#include <cuda_fp16.h>

namespace lbm {

struct pf2 {
  unsigned long long r;
  pf2() = default;
  __device__ __forceinline__ pf2(float a) { asm("mov.b64 %0, {%1, %1};" : "=l"(r) : "f"(a)); }
  __device__ __forceinline__ pf2(float a, float b) { asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b)); }
  __device__ __forceinline__ float lo() const {
    float a, b;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(r));
    return a;
  }
  __device__ __forceinline__ float hi() const {
    float a, b;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(r));
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

}  // namespace lbm
