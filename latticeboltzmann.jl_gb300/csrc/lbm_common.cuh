// lbm_common.cuh -- velocity sets, storage traits and kernel parameter blocks shared by the
// collide-stream kernels (lbm_step.cuh), the reductions (lbm_reduce.cuh) and the C ABI
// (lbm_api.cu).
#pragma once

#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <stdint.h>

#include <type_traits>

#include "../../include/lbm_gb300.h"
#include "lbm_df64.cuh"
#include "lbm_pf2.cuh"

namespace lbm {

// Compile-time loop: calls f(std::integral_constant<int, k>) for k = B .. E-1, so velocity and
// moment indices are constants inside the body and every lattice-table lookup, power and
// coefficient of the velocity set folds away.
template <int B, int E, class F>
__device__ __forceinline__ void static_for(F&& f) {
  if constexpr (B < E) {
    f(std::integral_constant<int, B>{});
    static_for<B + 1, E>(f);
  }
}

// Coordinates (x fastest) of the node numbers first, first + stride, ... of a grid-stride loop,
// with one 32-bit division at the start instead of a 64-bit division per node (lattices have
// fewer than 2^31 nodes, and strides are a grid's thread count).
struct NodeWalk {
  int x, y, sx, sy, nx;
  __device__ __forceinline__ NodeWalk(long long first, long long stride, int nx_) : nx(nx_) {
    const int n0 = (int)first, st = (int)stride;
    y = n0 / nx;
    x = n0 - y * nx;
    sy = st / nx;
    sx = st - sy * nx;
  }
  __device__ __forceinline__ void advance() {
    x += sx;
    y += sy;
    if (x >= nx) {
      x -= nx;
      ++y;
    }
  }
};

// Additions inside sums whose result feeds further arithmetic: plain for FP32 / FP64; for
// float-float without the closing renormalisation (add_lazy, lbm_df64.cuh).
template <class CT>
__device__ __forceinline__ CT ladd(CT a, CT b) { return a + b; }
template <class CT>
__device__ __forceinline__ CT lsub(CT a, CT b) { return a - b; }
#ifdef __CUDACC__
__device__ __forceinline__ dd ladd(dd a, dd b) { return add_lazy(a, b); }
__device__ __forceinline__ dd lsub(dd a, dd b) { return add_lazy(a, -b); }
#endif

// Multiply-add shapes c + a b, c - a b, a b + c, a b - c of the collision.  FP32 / FP64: explicit
// FMAs (below), so that which product is fused never depends on how often the compiler sees it
// used -- the same collision code then rounds alike whether it is inlined whole or split over
// warps (lbm_resident.cuh); float-float: lazy sums of products; packed FP32 pairs (lbm_pf2.cuh):
// one packed FMA.
template <class CT>
__device__ __forceinline__ CT add_prod(CT c, CT a, CT b) { return ladd(c, a * b); }
template <class CT>
__device__ __forceinline__ CT sub_prod(CT c, CT a, CT b) { return lsub(c, a * b); }
template <class CT>
__device__ __forceinline__ CT prod_add(CT a, CT b, CT c) { return ladd(a * b, c); }
template <class CT>
__device__ __forceinline__ CT prod_sub(CT a, CT b, CT c) { return lsub(a * b, c); }
// a b + c of a value that is stored (float-float: the normalised sum)
template <class CT>
__device__ __forceinline__ CT prod_add_out(CT a, CT b, CT c) { return a * b + c; }
#ifdef __CUDACC__
// FP32: explicit FMAs, so that one node (float) and two packed nodes (pf2) round alike
__device__ __forceinline__ float add_prod(float c, float a, float b) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ float sub_prod(float c, float a, float b) { return __fmaf_rn(-a, b, c); }
__device__ __forceinline__ float prod_add(float a, float b, float c) { return __fmaf_rn(a, b, c); }
// FP64: explicit FMAs as well
__device__ __forceinline__ double add_prod(double c, double a, double b) { return __fma_rn(a, b, c); }
__device__ __forceinline__ double sub_prod(double c, double a, double b) { return __fma_rn(-a, b, c); }
__device__ __forceinline__ double prod_add(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ double prod_sub(double a, double b, double c) { return __fma_rn(a, b, -c); }
__device__ __forceinline__ double prod_add_out(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float prod_sub(float a, float b, float c) { return __fmaf_rn(a, b, -c); }
__device__ __forceinline__ float prod_add_out(float a, float b, float c) { return __fmaf_rn(a, b, c); }
#endif

#ifdef __CUDACC__
// Programmatic dependent launch: a step kernel launched with programmatic stream serialization
// (launch_after_prior below) may be scheduled while the previous kernel on its stream still
// runs; it waits here, before touching global memory, until that kernel has completed and its
// writes are visible.  For a normal launch this is a no-op.
__device__ __forceinline__ void wait_prior_grid() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// A step kernel launched with programmatic stream serialization: it may be scheduled while the
// previous kernel on the stream finishes (it waits in wait_prior_grid before touching memory), so
// the launch latency between the back-to-back steps of a graph overlaps the previous step.
template <class... KArgs, class... Args>
inline void launch_after_prior(void (*kernel)(KArgs...), dim3 grid, dim3 block, cudaStream_t s, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}
#endif

// C t and v + C t for a compile-time integer C.  FP32 / FP64: a multiply and an FMA.  Float-float:
// the product of t with an exact integer skips the FMA of the zero trailing part that a general
// product spends, and for a power of two it is the exact scaling of both parts.
template <int C, class CT>
__device__ __forceinline__ CT mul_int(CT t) { return (CT)C * t; }
template <int C, class CT>
__device__ __forceinline__ CT add_int_prod(CT v, CT t) { return add_prod(v, (CT)C, t); }
#ifdef __CUDACC__
template <int C>
__device__ __forceinline__ dd mul_int(dd t) {
  constexpr int m = C < 0 ? -C : C;
  constexpr float c = (float)C;
  if constexpr ((m & (m - 1)) == 0) {
    return dd(__fmul_rn(t.hi, c), __fmul_rn(t.lo, c));
  } else {
    const float p = __fmul_rn(t.hi, c);
    return dd(p, __fmaf_rn(t.lo, c, __fmaf_rn(t.hi, c, -p)));
  }
}
template <int C>
__device__ __forceinline__ dd add_int_prod(dd v, dd t) { return add_lazy(v, mul_int<C>(t)); }
#endif

// v (+)= C t for a compile-time integer C; the first term initialises v, since IEEE arithmetic
// cannot fold a leading 0 + t away.  `set` is a constant at every point of an unrolled loop.
template <int C, class CT>
__device__ __forceinline__ void acc_add(CT& v, bool& set, CT t) {
  if constexpr (C == 1) {
    v = set ? ladd(v, t) : t;
    set = true;
  } else if constexpr (C == -1) {
    v = set ? lsub(v, t) : -t;
    set = true;
  } else if constexpr (C != 0) {
    v = set ? add_int_prod<C>(v, t) : mul_int<C>(t);
    set = true;
  }
}

// ---------------------------------------------------------------------------------------
// Velocity sets.  Abscissae and opposite maps as in src/quadratures/D2Q*.jl and
// src/quadratures.jl:11-19 (0-based).  The tables are compile-time so that every neighbour
// offset of the unrolled per-population loops folds to a register or an immediate.
//   R     : largest |c| component (halo radius of the pull)
//   EQ    : truncation order of `equilibrium!` (velocity_distribution_function/*.jl)
//   HN    : Hermite order of the regularised MRT, div(order(q), 2) (mrt.jl:68)
// ---------------------------------------------------------------------------------------
#define LBM_DEFINE_LATTICE(NAME, ID, QQ, RR, EQQ, HNN, CXS, CYS, OPS)                    \
  struct NAME {                                                                           \
    static constexpr int id = ID, Q = QQ, R = RR, EQ = EQQ, HN = HNN;                     \
    __host__ __device__ __forceinline__ static constexpr int cx(int i) {                  \
      constexpr int t[QQ] = CXS;                                                          \
      return t[i];                                                                        \
    }                                                                                     \
    __host__ __device__ __forceinline__ static constexpr int cy(int i) {                  \
      constexpr int t[QQ] = CYS;                                                          \
      return t[i];                                                                        \
    }                                                                                     \
    __host__ __device__ __forceinline__ static constexpr int opp(int i) {                 \
      constexpr int t[QQ] = OPS;                                                          \
      return t[i];                                                                        \
    }                                                                                     \
  };

#define LBM_L(...) {__VA_ARGS__}
LBM_DEFINE_LATTICE(D2Q4, 0, 4, 1, 1, 1, LBM_L(1, 0, -1, 0), LBM_L(0, 1, 0, -1), LBM_L(2, 3, 0, 1))
LBM_DEFINE_LATTICE(D2Q5, 1, 5, 1, 1, 1, LBM_L(0, 1, 0, -1, 0), LBM_L(0, 0, 1, 0, -1), LBM_L(0, 3, 4, 1, 2))
LBM_DEFINE_LATTICE(D2Q9, 2, 9, 1, 2, 2, LBM_L(0, -1, -1, -1, 0, 1, 1, 1, 0),
                   LBM_L(0, 1, 0, -1, -1, -1, 0, 1, 1), LBM_L(0, 5, 6, 7, 8, 1, 2, 3, 4))
LBM_DEFINE_LATTICE(D2Q13, 3, 13, 2, 2, 2, LBM_L(0, 1, -1, 0, 0, 1, -1, 1, -1, 2, -2, 0, 0),
                   LBM_L(0, 0, 0, 1, -1, 1, -1, -1, 1, 0, 0, -2, 2),
                   LBM_L(0, 2, 1, 4, 3, 6, 5, 8, 7, 10, 9, 12, 11))
LBM_DEFINE_LATTICE(D2Q17, 4, 17, 3, 3, 3, LBM_L(0, 1, -1, 0, 0, 1, -1, 1, -1, 2, -2, 2, -2, 3, -3, 0, 0),
                   LBM_L(0, 0, 0, 1, -1, 1, -1, -1, 1, 2, -2, -2, 2, 0, 0, 3, -3),
                   LBM_L(0, 2, 1, 4, 3, 6, 5, 8, 7, 10, 9, 12, 11, 14, 13, 16, 15))
LBM_DEFINE_LATTICE(D2Q21, 5, 25, 3, 3, 3,
                   LBM_L(0, 1, -1, 0, 0, 1, -1, 1, -1, 2, -2, 0, 0, 2, -2, 2, -2, 3, -3, 0, 0, 3, -3, -3, 3),
                   LBM_L(0, 0, 0, 1, -1, 1, -1, -1, 1, 0, 0, 2, -2, 2, -2, -2, 2, 0, 0, 3, -3, 3, -3, 3, -3),
                   LBM_L(0, 2, 1, 4, 3, 6, 5, 8, 7, 10, 9, 12, 11, 14, 13, 16, 15, 18, 17, 20, 19, 22, 21,
                         24, 23))
LBM_DEFINE_LATTICE(D2Q37, 6, 37, 3, 4, 4,
                   LBM_L(0, 1, -1, 0, 0, 1, -1, 1, -1, 2, -2, 0, 0, 2, -2, -2, 2, 1, -1, 1, -1, 2, -2, 2, -2,
                         3, -3, 0, 0, 3, -3, 3, -3, 1, -1, -1, 1),
                   LBM_L(0, 0, 0, 1, -1, 1, -1, -1, 1, 0, 0, 2, -2, 1, -1, 1, -1, 2, -2, -2, 2, 2, -2, -2, 2,
                         0, 0, 3, -3, 1, -1, -1, 1, 3, -3, 3, -3),
                   LBM_L(0, 2, 1, 4, 3, 6, 5, 8, 7, 10, 9, 12, 11, 14, 13, 16, 15, 18, 17, 20, 19, 22, 21,
                         24, 23, 26, 25, 28, 27, 30, 29, 32, 31, 34, 33, 36, 35))
#undef LBM_L

// ---------------------------------------------------------------------------------------
// Storage traits.  F64 stores f; F32Dev / F16Dev store g = f - w and compute in FP32.
// ---------------------------------------------------------------------------------------
struct F64 {
  using T = double;     // element in HBM
  using C = double;     // compute type
  static constexpr bool DEV = false;
  static constexpr bool SR = false;    // collision outputs stored with stochastic rounding
  static constexpr bool WIDE = false;  // stores f but computes on g = f - w (F64DD)
  static constexpr int id = LBM_STORE_F64;
  __device__ __forceinline__ static C ld(const T* p) { return __ldg(p); }
  __device__ __forceinline__ static void st(T* p, C v) { *p = v; }
};
// ld2 / st2: the values of two x-adjacent nodes as one aligned access (p at an even element).
struct F32Dev {
  using T = float;
  using C = float;
  static constexpr bool DEV = true;
  static constexpr bool SR = false;
  static constexpr bool WIDE = false;
  static constexpr int id = LBM_STORE_F32_DEV;
  __device__ __forceinline__ static C ld(const T* p) { return __ldg(p); }
  __device__ __forceinline__ static void st(T* p, C v) { *p = v; }
  __device__ __forceinline__ static pf2 ld2(const T* p) {
    pf2 v;
    v.r = __ldg(reinterpret_cast<const unsigned long long*>(p));
    return v;
  }
  __device__ __forceinline__ static void st2(T* p, pf2 v) { *reinterpret_cast<unsigned long long*>(p) = v.r; }
};
struct F16Dev {
  using T = __half;
  using C = float;
  static constexpr bool DEV = true;
  static constexpr bool SR = false;
  static constexpr bool WIDE = false;
  static constexpr int id = LBM_STORE_F16_DEV;
  __device__ __forceinline__ static C ld(const T* p) { return __half2float(__ldg(p)); }
  __device__ __forceinline__ static void st(T* p, C v) { *p = __float2half_rn(v); }
  __device__ __forceinline__ static pf2 ld2(const T* p) {
    const float2 f = __half22float2(__ldg(reinterpret_cast<const __half2*>(p)));
    return pf2(f.x, f.y);
  }
  __device__ __forceinline__ static void st2(T* p, pf2 v) {
    *reinterpret_cast<__half2*>(p) = __floats2half2_rn(v.lo(), v.hi());
  }
};

struct DF64Dev {
  using T = float2;
  using C = dd;
  static constexpr bool DEV = true;
  static constexpr bool SR = false;
  static constexpr bool WIDE = false;
  static constexpr int id = LBM_STORE_DF64_DEV;
  __device__ __forceinline__ static C ld(const T* p) {
    const float2 v = __ldg(p);
    return dd(v.x, v.y);
  }
  __device__ __forceinline__ static void st(T* p, C v) { *p = make_float2(v.hi, v.lo); }
  __device__ __forceinline__ static pdd ld2(const T* p) {
    const float4 v = __ldg(reinterpret_cast<const float4*>(p));
    return pdd(pf2(v.x, v.z), pf2(v.y, v.w));
  }
  __device__ __forceinline__ static void st2(T* p, pdd v) {
    *reinterpret_cast<float4*>(p) = make_float4(v.hi.lo(), v.lo.lo(), v.hi.hi(), v.lo.hi());
  }
};

// FP32 deviation storage computed in float-float arithmetic, whose collision outputs are stored
// with stochastic rounding (st_sr): the float-float value hi + lo becomes hi, or hi's neighbour
// towards lo, with probability |lo| / (distance to that neighbour), so the stored value is the
// exact one in expectation.  With round-to-nearest, a small increment (a body force of 1e-6 on
// deviations of 1e-3) that meets near-identical values every step rounds the same way every step
// and the error grows linearly in time; unbiased rounding leaves a random walk, which diffusion
// spreads and averages.  Everything else (uploads, the pull without collision) rounds to nearest.
struct F32DevSR {
  using T = float;
  using C = dd;
  static constexpr bool DEV = true;
  static constexpr bool SR = true;
  static constexpr bool WIDE = false;
  static constexpr int id = LBM_STORE_F32_DEV_SR;
  __device__ __forceinline__ static C ld(const T* p) { return dd(__ldg(p), 0.f); }
  __device__ __forceinline__ static void st(T* p, C v) { *p = __fadd_rn(v.hi, v.lo); }
  __device__ __forceinline__ static pdd ld2(const T* p) {
    pf2 v;
    v.r = __ldg(reinterpret_cast<const unsigned long long*>(p));
    return pdd(v, pf2(0.f));
  }
};

// 32 uniform bits from (node, population, step): the three are mixed by odd multipliers and the
// result goes through the "lowbias32" integer finaliser (xor-shift / multiply rounds with the
// constants C. Wellons published for it).  Counter-based, so a run is reproducible.
__device__ __forceinline__ unsigned sr_bits(unsigned node, unsigned pop, unsigned step) {
  unsigned h = node * 0x9E3779B9u ^ (pop + 1u) * 0x85EBCA6Bu ^ (step + 0x632BE5ABu) * 0xC2B2AE35u;
  h ^= h >> 16;
  h *= 0x7FEB352Du;
  h ^= h >> 15;
  h *= 0x846CA68Bu;
  h ^= h >> 16;
  return h;
}

// Stochastic rounding of a normalised float-float value (|lo| at most half an ulp of hi) to a
// float, with the uniform bits h: the neighbour n of hi towards lo is taken when u |n - hi| < |lo|,
// u in [0, 1) the top 23 bits of h (formed from the bits, as 1.f..2.f minus one: no integer-to-float
// conversion).  |n - hi| is a power of two, so the product and the comparison are exact.
__device__ __forceinline__ float round_stochastic(float hi, float lo, unsigned h) {
  if (lo == 0.f || hi == 0.f || !isfinite(hi)) return __fadd_rn(hi, lo);
  const int b = __float_as_int(hi);
  const float n = __int_as_float(b + (((lo > 0.f) == (hi > 0.f)) ? 1 : -1));
  const float gap = fabsf(__fsub_rn(n, hi));
  const float u = __fsub_rn(__int_as_float(0x3F800000u | (h >> 9)), 1.0f);
  return __fmul_rn(u, gap) < fabsf(lo) ? n : hi;
}

// FP64 storage (f itself, the reference's bytes) with float-float arithmetic on the deviation
// g = f - w.  On this GPU a double <-> float conversion instruction runs at the FP64 rate, as slow as
// the FP64 arithmetic it would replace, so the splits are made with integer operations: a load
// forms g = f - w with one FP64 subtraction and splits it into a float-float pair from its bits; a
// store rebuilds the doubles of hi and lo from their bits and forms w + (hi + lo) with two FP64
// additions (hi + lo is exact in FP64 when lo lies within 29 bits of hi, as the collision's
// normalised outputs do, and rounds once otherwise).  The collision is the float-float one of
// DF64Dev, so a value carries 48 bits on the deviation, below FP64's own rounding of f.
struct F64DD {
  using T = double;
  using C = dd;
  static constexpr bool DEV = true;
  static constexpr bool SR = false;
  static constexpr bool WIDE = true;
  static constexpr int id = LBM_STORE_F64_DD;
  // x as hi + lo: hi the top 24 significand bits of x (truncated), lo the next 29 rounded to the
  // nearest float, renormalised.  Integer and FP32 instructions only, with no branch to a
  // conversion: on this GPU a double-float conversion, an integer-to-float conversion and a 64-bit
  // integer operation all issue to the FP64 pipe, where even a predicated-off instruction takes
  // its slot.  Every bit operation is on the two 32-bit words of x.  Range: |x| >= 2^-74 splits
  // exactly as stated; for 2^-126 <= |x| < 2^-74 lo is flushed to zero (absolute error below
  // 2^-98); smaller |x| (double subnormals and zero) give a signed zero; |x| >= 2^128 gives an
  // infinity and a NaN stays a NaN.
  __device__ __forceinline__ static dd split(double x) {
    const unsigned hw = (unsigned)__double2hiint(x), lw = (unsigned)__double2loint(x);
    const int e = (int)((hw >> 20) & 0x7FFu);
    const unsigned sgn = hw & 0x80000000u;
    const float hi = __uint_as_float(sgn | ((unsigned)(e - 896) << 23) | ((hw & 0xFFFFFu) << 3) | (lw >> 29));
    // lo = r 2^(e - 1075) for the 29 bits r below hi's: r's top 23 and low 6 bits become exact
    // floats through the 2^23 exponent trick, one FMA joins them (rounding to 24 bits) and the
    // power-of-two scale places them; the scale is zero (lo flushed) for e < 949
    const unsigned r = lw & 0x1FFFFFFFu;
    const float ra = __fsub_rn(__uint_as_float(0x4B000000u | (r >> 6)), 8388608.f);
    const float rb = __fsub_rn(__uint_as_float(0x4B000000u | (r & 63u)), 8388608.f);
    const float scale = __uint_as_float((unsigned)max(e - 948, 0) << 23);
    const float lo = __uint_as_float(__float_as_uint(__fmul_rn(__fmaf_rn(ra, 64.f, rb), scale)) | sgn);
    const dd out = fast_two_sum(hi, lo);
    const bool nan = e == 2047 && ((hw & 0xFFFFFu) | lw) != 0u;
    const unsigned special = e < 897 ? sgn : (nan ? 0x7FC00000u : (sgn | 0x7F800000u));
    const bool normal = e >= 897 && e <= 1150;
    return dd(normal ? out.hi : __uint_as_float(special), normal ? out.lo : 0.f);
  }
  // the double of a normalised pair hi + lo (|lo| <= ulp(hi) / 2, as every float-float addition
  // leaves it), assembled from the bits: hi's significand times 2^29 plus lo's significand aligned
  // to the same units, lo rounded half away from zero where its last bits fall below them (error
  // at most 2^-52 |hi + lo|).  A zero or float-subnormal hi gives a signed zero and a
  // float-subnormal lo is dropped (absolute error below 2^-126 either way); an infinite or NaN hi
  // stays one.
  __device__ __forceinline__ static double widen2(float h, float l) {
    const unsigned uh = __float_as_uint(h), ul = __float_as_uint(l);
    const int eh = (int)((uh >> 23) & 0xFFu), el = (int)((ul >> 23) & 0xFFu);
    const unsigned mh = (uh & 0x7FFFFFu) | 0x800000u, ml = (ul & 0x7FFFFFu) | 0x800000u;
    // L = lo / 2^(eh - 179) rounded, < 2^29: d = eh - el >= 24 for a normalised pair
    const int d = eh - el;
    const int sr = min(max(d - 29, 1), 31);
    const unsigned down_l = d <= 29 ? (ml << (29 - d)) : ((ml + (1u << (sr - 1))) >> sr);
    const unsigned L = (el == 0 || d > 53) ? 0u : down_l;
    const unsigned a_hi = mh >> 3, a_lo = mh << 29;
    unsigned r_hi, r_lo;
    if (((uh ^ ul) & 0x80000000u) == 0u) {
      r_hi = a_hi;
      r_lo = a_lo | L;
    } else {
      r_hi = a_hi - (L > a_lo ? 1u : 0u);
      r_lo = a_lo - L;
    }
    // a subtraction from a power-of-two hi can borrow the leading bit: shift it back into place
    const unsigned dn = r_hi < 0x100000u ? 1u : 0u;
    r_hi = dn ? ((r_hi << 1) | (r_lo >> 31)) : r_hi;
    r_lo = r_lo << dn;
    const unsigned sgn = uh & 0x80000000u;
    const unsigned word = eh == 0 ? sgn
                        : (eh == 255 ? (sgn | 0x7FF00000u | ((uh & 0x7FFFFFu) ? 0x80000u : 0u))
                                     : (sgn | ((unsigned)(eh + 896 - (int)dn) << 20) | (r_hi & 0xFFFFFu)));
    const unsigned lword = (eh == 0 || eh == 255) ? 0u : r_lo;
    return __hiloint2double((int)word, (int)lword);
  }
  __device__ __forceinline__ static C from_f(double f, double w) { return split(__dsub_rn(f, w)); }
  // collision outputs may be unnormalised pairs (a product's (p, e), |e| well below |p|): one
  // fast two-sum normalises them for widen2
  __device__ __forceinline__ static double to_f(C g, double w) {
    const dd n = fast_two_sum(g.hi, g.lo);
    return __dadd_rn(w, widen2(n.hi, n.lo));
  }
};

// ---------------------------------------------------------------------------------------
// Kernel parameter blocks (passed by value; they live in the constant bank).
// ---------------------------------------------------------------------------------------
struct BCDev {
  int kind, dir;
  int x_lo, x_hi, y_lo, y_hi;  // 0-based inclusive
  double add[LBM_MAX_Q];       // MOVING_WALL: 2 * a_1 per population (moving_wall.jl:20-33)
};

template <class CT>
struct StepParams {
  int nx, ny;
  long long n;                 // plane stride nx * ny
  int dxm[7], dym[7];          // (d mod nx), (d mod ny) for d = -3..3 (periodic pull offsets)
  CT w[LBM_MAX_Q];
  CT cs;                       // 1 / c_s^2 (the reference's speed_of_sound_squared)
  CT om_a, om_b;               // SRT: (1 - 1/τ), 1/τ ; ITER: same
  CT inv_ts, inv_ta;           // TRT: 1/τ_s, 1/τ_a
  CT shift;                    // force velocity shift: τ (SRT), τ_a (TRT), τs[2] (MRT)
  CT pa_s, pa_a, pom_s, pom_a; // pair form: (1 - ω_s)/2, (1 - ω_a)/2, ω_s, ω_a (SRT: ω_s = ω_a = 1/τ)
  CT hcs, hcs2;                // pair form: (1/c_s²)/2, (1/c_s²)²/2
  CT pws[LBM_MAX_Q];           // pair form: ω_s w_i
  CT pwa[LBM_MAX_Q];           // pair form: ω_a w_i
  CT pw1a[LBM_MAX_Q];          // pair form: ω_a w1_i
  CT pa_s2;                    // pair form: 1 - ω_s (rest population)
  CT sF[2];                    // CONSTANT force times the velocity shift
  CT w1[LBM_MAX_Q];            // deviation storage: first-order equilibrium coefficients (1/c_s²)·w_i,
                               // chosen so that Σ_i w1_i c_ix² = 1 holds for the values as stored
  CT mrt_a[4], mrt_b[4];       // MRT: (1 - 1/τ_n), 1/τ_n for n = 1..4
  int force_kind;
  CT F[2];                     // CONSTANT force
  const double* Ffield;        // FIELD force planes (device)
  double shear[6];             // SHEAR force
  const double* xr;            // SHEAR coordinates (device)
  const double* yr;
  double time;                 // physical time of this step
  const long long* time_base;  // when set: {t0, bits of Δt} on the device, and the step runs at
  int time_step;               // time (t0 + time_step) Δt (steps of a CUDA graph, see step_time)
  long long step_index;        // time index of this step when time_base is not set (the counter of
                               // stochastic rounding, step_counter)
  double wf[LBM_MAX_Q];        // the weights in FP64 (F64DD: f = w + g on load and store)
  const CT* nonlinear;         // ITER: nonlinear equilibrium term planes (device)
  int nbc;
  BCDev bc[LBM_MAX_BC];
};

}  // namespace lbm
