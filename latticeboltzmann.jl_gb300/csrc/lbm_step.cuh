// lbm_step.cuh -- the fused collide-stream kernels.
//
// One time step of the reference loop (src/lattice_boltzmann_model.jl:64-67)
//     collide!  ->  stream! (periodic pull, stream.jl:18-30)  ->  apply!(bcs)
// is issued as ONE kernel over the lattice.  The device keeps the post-collision array of
// the previous step; a step pulls the streamed populations of every node from it (with
// the boundary conditions overriding the populations whose pull source lies outside the
// wall), collides them and writes the node's new post-collision populations.  The first
// step after an upload runs the collision alone, and the state the reference exposes as
// `f_stream` is obtained on demand by the pull without the collision.
//
// Layout in HBM: the reference's Julia array f[x, y, i], i.e. Q planes of nx*ny values,
// x fastest.  A warp covers 32 consecutive x of one row, so each population plane is read
// and written as coalesced 32-wide segments (shifted by c_ix for the pull).
#pragma once

#include "lbm_common.cuh"

namespace lbm {

// Offset of population plane i: a 32 x 32 -> 64-bit product, since lattices have fewer than 2^31
// nodes (lbm_create checks), so that a population's address costs two wide multiply-adds instead
// of 64-bit multiply arithmetic.
template <class CT>
__device__ __forceinline__ size_t plane_off(const StepParams<CT>& p, int i) {
  return (size_t)(unsigned)p.n * (unsigned)i;
}

// Population i at `ptr` in the compute type, and its store: S::ld / S::st, except for a storage
// that keeps f itself but computes on the deviation (F64DD), which forms g = f - w on load and
// w + g on store with the FP64 weight.
template <class S, class CT>
__device__ __forceinline__ typename S::C load_pop(const StepParams<CT>& p, const typename S::T* ptr, int i) {
  if constexpr (S::WIDE) return S::from_f(__ldg(ptr), p.wf[i]);
  else return S::ld(ptr);
}
template <class S, class CT>
__device__ __forceinline__ void store_pop(const StepParams<CT>& p, typename S::T* ptr, int i, typename S::C v) {
  if constexpr (S::WIDE) *ptr = S::to_f(v, p.wf[i]);
  else S::st(ptr, v);
}

// Periodic pull offsets: xw[k] = (x - (k - R)) mod nx, yo[k] = ((y - (k - R)) mod ny) * nx.
template <class L, class CT>
__device__ __forceinline__ void pull_offsets(const StepParams<CT>& p, int x, int y, int* xw, int* yo) {
#pragma unroll
  for (int k = 0; k < 2 * L::R + 1; ++k) {
    const int d = k - L::R;
    int xs = x - p.dxm[d + 3];
    xs += (xs < 0) ? p.nx : 0;
    xw[k] = xs;
    int ys = y - p.dym[d + 3];
    ys += (ys < 0) ? p.ny : 0;
    yo[k] = ys * p.nx;
  }
}

// Streamed populations of node (x, y): the periodic pull of stream!, then the boundary
// conditions in list order (bounce_back.jl:8-72, moving_wall.jl:17-38), which overwrite a
// population with the same node's post-collision value of the opposite population.
template <class L, class S, class CT>
__device__ __forceinline__ void load_streamed(const StepParams<CT>& p, const typename S::T* __restrict__ src,
                                              int x, int y, typename S::C* f) {
  int xw[2 * L::R + 1], yo[2 * L::R + 1];
  pull_offsets<L>(p, x, y, xw, yo);
#pragma unroll
  for (int i = 0; i < L::Q; ++i) {
    const int idx = yo[L::R + L::cy(i)] + xw[L::R + L::cx(i)];
    f[i] = load_pop<S>(p, src + plane_off(p, i) + idx, i);
  }
  if (p.nbc > 0 &&
      (y < L::R || y >= p.ny - L::R || x < L::R || x >= p.nx - L::R)) {
    const int node = y * p.nx + x;
    const int y1 = y + 1, x1 = x + 1;  // the reference's 1-based indices
    for (int b = 0; b < p.nbc; ++b) {
      const BCDev& bc = p.bc[b];
      if (bc.kind == LBM_BOUNCE_BACK) {
        if (x < bc.x_lo || x > bc.x_hi || y < bc.y_lo || y > bc.y_hi) continue;
#pragma unroll
        for (int i = 0; i < L::Q; ++i) {
          const int o = L::opp(i);
          bool hit;
          if (bc.dir == LBM_NORTH) hit = y1 + L::cy(o) > p.ny;
          else if (bc.dir == LBM_SOUTH) hit = y1 + L::cy(o) <= 0;
          else if (bc.dir == LBM_EAST) hit = x1 + L::cx(o) > p.nx;
          else hit = x1 + L::cx(o) <= 0;
          if (hit) f[i] = load_pop<S>(p, src + plane_off(p, o) + node, o);
        }
      } else {  // MovingWall{North}: whole top wall, ignores xs / ys
#pragma unroll
        for (int i = 0; i < L::Q; ++i) {
          const int o = L::opp(i);
          if (y1 + L::cy(o) > p.ny) f[i] = load_pop<S>(p, src + plane_off(p, o) + node, o) + (typename S::C)bc.add[i];
        }
      }
    }
  }
}

// Population i of node (x, y) after the pull and the boundary rules, one population at a time
// (for kernels that consume populations as they arrive instead of holding all Q).
template <class L, class S, class CT>
__device__ __forceinline__ typename S::C pop_streamed(const StepParams<CT>& p, const typename S::T* __restrict__ src,
                                                      int x, int y, const int* xw, const int* yo, bool near, int i) {
  typename S::C v = load_pop<S>(p, src + plane_off(p, i) + yo[L::R + L::cy(i)] + xw[L::R + L::cx(i)], i);
  if (near) {
    const int node = y * p.nx + x;
    const int y1 = y + 1, x1 = x + 1;
    const int o = L::opp(i);
    for (int b = 0; b < p.nbc; ++b) {
      const BCDev& bc = p.bc[b];
      if (bc.kind == LBM_BOUNCE_BACK) {
        if (x < bc.x_lo || x > bc.x_hi || y < bc.y_lo || y > bc.y_hi) continue;
        bool hit;
        if (bc.dir == LBM_NORTH) hit = y1 + L::cy(o) > p.ny;
        else if (bc.dir == LBM_SOUTH) hit = y1 + L::cy(o) <= 0;
        else if (bc.dir == LBM_EAST) hit = x1 + L::cx(o) > p.nx;
        else hit = x1 + L::cx(o) <= 0;
        if (hit) v = load_pop<S>(p, src + plane_off(p, o) + node, o);
      } else if (y1 + L::cy(o) > p.ny) {
        v = load_pop<S>(p, src + plane_off(p, o) + node, o) + (typename S::C)bc.add[i];
      }
    }
  }
  return v;
}

template <class L, class S, class CT>
__device__ __forceinline__ void load_local(const StepParams<CT>& p, const typename S::T* __restrict__ src,
                                           int node, typename S::C* f) {
#pragma unroll
  for (int i = 0; i < L::Q; ++i) f[i] = load_pop<S>(p, src + plane_off(p, i) + node, i);
}

// Physical time of the step: p.time, or, for the steps of a captured CUDA graph of a lattice with a
// time-dependent force, (t0 + time_step) Δt with t0 and Δt written to the device before each
// graph launch -- the same product of the same doubles as the host's (t0 + k) Δt.
template <class CT>
__device__ __forceinline__ double step_time(const StepParams<CT>& p) {
  if (!p.time_base) return p.time;
  return (double)(p.time_base[0] + p.time_step) * __longlong_as_double(p.time_base[1]);
}

// Counter of the stochastic rounding of SR storages: the time index of the step (the graph's t0 +
// its step number, or the index the host set for an eager launch).
template <class CT>
__device__ __forceinline__ unsigned step_counter(const StepParams<CT>& p) {
  return (unsigned)(p.time_base ? p.time_base[0] + p.time_step : p.step_index);
}

// Stores collision output i of node `node`: stochastically rounded for an SR storage (F32DevSR),
// else as S::st.
template <class S, class CT>
__device__ __forceinline__ void store_out(const StepParams<CT>& p, typename S::T* dst, int i, int node,
                                          typename S::C v) {
  if constexpr (S::SR) dst[plane_off(p, i) + node] = round_stochastic(v.hi, v.lo, sr_bits(node, i, step_counter(p)));
  else store_pop<S>(p, dst + plane_off(p, i) + node, i, v);
}

// Lattice force at node (x, y), lattice_force(problem, x, y, t) (problems.jl:103-104).  `time()`
// gives the physical time of the step; it is called only for the time-dependent force, so the
// steps of the other forces spend no FP64 instruction on it.
template <class CT, class TimeFn>
__device__ __forceinline__ void node_force(const StepParams<CT>& p, int x, int y, CT& Fx, CT& Fy, TimeFn&& time) {
  if (p.force_kind == LBM_FORCE_CONSTANT) {
    Fx = p.F[0];
    Fy = p.F[1];
  } else if (p.force_kind == LBM_FORCE_FIELD) {
    const size_t k = (size_t)y * p.nx + x;
    Fx = (CT)__ldg(p.Ffield + k);
    Fy = (CT)__ldg(p.Ffield + p.n + k);
  } else if (p.force_kind == LBM_FORCE_SHEAR) {
    const double X = __ldg(p.xr + x), Y = __ldg(p.yr + y), t = time();
    Fx = (CT)(p.shear[0] * cos(p.shear[1] * Y - p.shear[2] * t));
    Fy = (CT)(p.shear[3] * cos(p.shear[4] * X - p.shear[5] * t));
  } else {
    Fx = 0;
    Fy = 0;
  }
}
// Lattice force at node (x, y) times the velocity shift (τ for SRT, τ_a for TRT, τ_2 for MRT),
// i.e. the term the collision adds to u; for a CONSTANT force the product comes from the host.
template <class CT, class TimeFn>
__device__ __forceinline__ void node_shifted_force(const StepParams<CT>& p, int x, int y, CT& sFx, CT& sFy,
                                                   TimeFn&& time) {
  if (p.force_kind == LBM_FORCE_CONSTANT) {
    sFx = p.sF[0];
    sFy = p.sF[1];
  } else {
    CT Fx, Fy;
    node_force(p, x, y, Fx, Fy, time);
    sFx = p.shift * Fx;
    sFy = p.shift * Fy;
  }
}

// `equilibrium!` truncation by velocity set: first order (D2Q4/5), second (D2Q9/13), third
// (D2Q17/21), fourth (D2Q37).  Returns the bracket 1 + a1 + a2/2 [+ a3/6 + a4/24] minus 1,
// so that feq_i = ρ w_i (1 + P_i).
template <class L, class CT>
__device__ __forceinline__ CT eq_poly_hi(CT cs, CT cu, CT usq) {  // the terms of order >= 2
  if constexpr (L::EQ == 1) {
    return (CT)0;
  } else {
    const CT cs2 = cs * cs;
    const CT cu2 = cu * cu;
    const CT a2 = cs2 * cu2 - cs * usq;
    CT r = (CT)0.5 * a2;
    if constexpr (L::EQ >= 3) {
      const CT a3 = (cs * cu) * (cs2 * cu2 - ((CT)3 * cs) * usq);
      r += (CT)(1.0 / 6.0) * a3;
    }
    if constexpr (L::EQ >= 4) {
      const CT a4 = (cs2 * cs2) * (cu2 * cu2) - (((CT)6 * (cs2 * cs)) * usq) * cu2 + ((CT)3 * cs2) * (usq * usq);
      r += (CT)(1.0 / 24.0) * a4;
    }
    return r;
  }
}

template <class L, class CT>
__device__ __forceinline__ CT eq_poly(CT cs, CT cu, CT usq) {
  const CT a1 = cs * cu;
  if constexpr (L::EQ == 1) return a1;
  else return a1 + eq_poly_hi<L>(cs, cu, usq);
}

// Raw moments M_ab = Σ_i v_i cx_i^a cy_i^b, a + b <= 4, in the order
// 00, 10, 01, 20, 11, 02, 30, 21, 12, 03, 40, 31, 22, 13, 04.
__host__ __device__ constexpr int mom_a(int k) {
  return k == 0 ? 0 : k == 1 ? 1 : k == 2 ? 0 : k == 3 ? 2 : k == 4 ? 1 : k == 5 ? 0 : k == 6 ? 3 : k == 7 ? 2
       : k == 8 ? 1 : k == 9 ? 0 : k == 10 ? 4 : k == 11 ? 3 : k == 12 ? 2 : k == 13 ? 1 : 0;
}
__host__ __device__ constexpr int mom_b(int k) {
  return k == 0 ? 0 : k == 1 ? 0 : k == 2 ? 1 : k == 3 ? 0 : k == 4 ? 1 : k == 5 ? 2 : k == 6 ? 0 : k == 7 ? 1
       : k == 8 ? 2 : k == 9 ? 3 : k == 10 ? 0 : k == 11 ? 1 : k == 12 ? 2 : k == 13 ? 3 : 4;
}
__host__ __device__ constexpr int ipow(int c, int e) { return e == 0 ? 1 : c * ipow(c, e - 1); }
__host__ __device__ constexpr int mom_count(int hn) { return hn <= 1 ? 3 : hn == 2 ? 6 : hn == 3 ? 10 : 15; }

template <class CT>
struct MrtCoeffs {
  CT B[15];      // coefficients of the monomials c_x^a c_y^b of f_out / w
  CT B1p, B2p;   // deviation storage: first-order coefficients per w1 = c w
};

// Raw moments accumulated pair by pair: opposite populations I, opp(I) enter through
// s = f_I + f_opp and d = f_I - f_opp, since c_opp = -c_I flips every monomial of odd degree.
template <class L, int I, class CT>
__device__ __forceinline__ void mrt_accumulate_pair(CT* M, bool* set, CT s, CT d) {
  static_for<0, mom_count(L::HN)>([&](auto K) {
    constexpr int k = decltype(K)::value;
    constexpr int coef = ipow(L::cx(I), mom_a(k)) * ipow(L::cy(I), mom_b(k));
    acc_add<coef>(M[k], set[k], ((mom_a(k) + mom_b(k)) & 1) ? d : s);
  });
}

// Relaxation of the Hermite coefficients from the raw moments M (see mrt_collide).
template <class L, bool DEV, class CT>
__device__ __forceinline__ void mrt_coeffs(const StepParams<CT>& p, const CT* M, CT sFx, CT sFy, bool has_force,
                                           MrtCoeffs<CT>& c) {
  const CT rho = DEV ? ladd((CT)1, M[0]) : M[0];
  const CT inv_rho = (CT)1 / rho;
  CT ux = M[1] * inv_rho, uy = M[2] * inv_rho;
  if (has_force) {
    ux = ladd(ux, sFx);
    uy = ladd(uy, sFy);
  }
  const CT cs = p.cs, ics = (CT)1 / cs;  // ics = c_s^2
  CT* B = c.B;  // every coefficient is assigned before it is updated (no 0 + x)
  B[0] = M[0];  // ρ, or ρ - 1 in deviation form
  B[1] = cs * rho * ux;
  B[2] = cs * rho * uy;
  c.B1p = rho * ux;
  c.B2p = rho * uy;
  if constexpr (L::HN >= 2) {
    const CT a = p.mrt_a[1], b = p.mrt_b[1];
    const CT Axx = ladd(a * lsub(M[3], ics * M[0]), b * (rho * ux * ux));
    const CT Axy = ladd(a * M[4], b * (rho * ux * uy));
    const CT Ayy = ladd(a * lsub(M[5], ics * M[0]), b * (rho * uy * uy));
    const CT c2 = cs * cs * (CT)0.5;
    B[3] = c2 * Axx;
    B[4] = c2 * (CT)2 * Axy;
    B[5] = c2 * Ayy;
    B[0] = lsub(B[0], c2 * ics * ladd(Axx, Ayy));
  }
  if constexpr (L::HN >= 3) {
    const CT a = p.mrt_a[2], b = p.mrt_b[2];
    const CT Axxx = ladd(a * lsub(M[6], (CT)3 * ics * M[1]), b * (rho * ux * ux * ux));
    const CT Axxy = ladd(a * lsub(M[7], ics * M[2]), b * (rho * ux * ux * uy));
    const CT Axyy = ladd(a * lsub(M[8], ics * M[1]), b * (rho * ux * uy * uy));
    const CT Ayyy = ladd(a * lsub(M[9], (CT)3 * ics * M[2]), b * (rho * uy * uy * uy));
    const CT c3 = cs * cs * cs * (CT)(1.0 / 6.0);
    B[6] = c3 * Axxx;
    B[7] = c3 * (CT)3 * Axxy;
    B[8] = c3 * (CT)3 * Axyy;
    B[9] = c3 * Ayyy;
    const CT sx = ladd(Axxx, Axyy), sy = ladd(Axxy, Ayyy);
    B[1] = lsub(B[1], c3 * (CT)3 * ics * sx);
    B[2] = lsub(B[2], c3 * (CT)3 * ics * sy);
    c.B1p = lsub(c.B1p, c3 * (CT)3 * ics * ics * sx);
    c.B2p = lsub(c.B2p, c3 * (CT)3 * ics * ics * sy);
  }
  if constexpr (L::HN >= 4) {
    const CT a = p.mrt_a[3], b = p.mrt_b[3];
    const CT ics2 = ics * ics;
    const CT Axxxx = ladd(a * ladd(lsub(M[10], (CT)6 * ics * M[3]), (CT)3 * ics2 * M[0]), b * (rho * ux * ux * ux * ux));
    const CT Axxxy = ladd(a * lsub(M[11], (CT)3 * ics * M[4]), b * (rho * ux * ux * ux * uy));
    const CT Axxyy = ladd(a * ladd(lsub(M[12], ics * ladd(M[3], M[5])), ics2 * M[0]), b * (rho * ux * ux * uy * uy));
    const CT Axyyy = ladd(a * lsub(M[13], (CT)3 * ics * M[4]), b * (rho * ux * uy * uy * uy));
    const CT Ayyyy = ladd(a * ladd(lsub(M[14], (CT)6 * ics * M[5]), (CT)3 * ics2 * M[0]), b * (rho * uy * uy * uy * uy));
    const CT c4 = cs * cs * cs * cs * (CT)(1.0 / 24.0);
    B[10] = c4 * Axxxx;
    B[11] = c4 * (CT)4 * Axxxy;
    B[12] = c4 * (CT)6 * Axxyy;
    B[13] = c4 * (CT)4 * Axyyy;
    B[14] = c4 * Ayyyy;
    B[3] = lsub(B[3], c4 * ics * (CT)6 * ladd(Axxxx, Axxyy));
    B[4] = lsub(B[4], c4 * ics * (CT)12 * ladd(Axxxy, Axyyy));
    B[5] = lsub(B[5], c4 * ics * (CT)6 * ladd(Axxyy, Ayyyy));
    B[0] = ladd(B[0], c4 * ics2 * ladd(ladd((CT)3 * Axxxx, (CT)6 * Axxyy), (CT)3 * Ayyyy));
  }
}

// Post-collision pair I, opp(I) rebuilt from the coefficients: the even- and odd-degree parts
// E, O of population I give f_I = w (E + O) and f_opp = w (E - O).  Deviation storage: the
// first-order monomials carry w1_I / c instead of w_I (see collide_pairs).
template <class L, bool DEV, int I, class CT>
__device__ __forceinline__ void mrt_out_pair(const StepParams<CT>& p, const MrtCoeffs<CT>& c, CT& out_i, CT& out_o) {
  CT E = c.B[0], O;
  bool se = true, so = false;
  static_for<(DEV ? 3 : 1), mom_count(L::HN)>([&](auto K) {
    constexpr int k = decltype(K)::value;
    constexpr int coef = ipow(L::cx(I), mom_a(k)) * ipow(L::cy(I), mom_b(k));
    if constexpr ((mom_a(k) + mom_b(k)) & 1) acc_add<coef>(O, so, c.B[k]);
    else acc_add<coef>(E, se, c.B[k]);
  });
  const CT we = p.w[I] * E;
  CT wo = so ? p.w[I] * O : (CT)0;
  if constexpr (DEV) {
    CT s1;
    bool s1s = false;
    acc_add<L::cx(I)>(s1, s1s, c.B1p);
    acc_add<L::cy(I)>(s1, s1s, c.B2p);
    wo = so ? ladd(wo, p.w1[I] * s1) : p.w1[I] * s1;
  }
  out_i = we + wo;
  out_o = we - wo;
}

// Index of the velocity (cx, cy) in set L, or -1.
template <class L>
__host__ __device__ constexpr int vel_index(int cx, int cy) {
  for (int j = 0; j < L::Q; ++j)
    if (L::cx(j) == cx && L::cy(j) == cy) return j;
  return -1;
}

// Velocity i with both components positive heads the quadruple {(a, b), (a, -b), (-a, b), (-a, -b)}.
template <class L>
__host__ __device__ constexpr bool quad_head(int i) {
  return L::cx(i) > 0 && L::cy(i) > 0 && vel_index<L>(L::cx(i), -L::cy(i)) >= 0 &&
         vel_index<L>(-L::cx(i), L::cy(i)) >= 0;
}
template <class L>
__host__ __device__ constexpr bool in_quad(int i) {
  const int a = L::cx(i) < 0 ? -L::cx(i) : L::cx(i), b = L::cy(i) < 0 ? -L::cy(i) : L::cy(i);
  return a > 0 && b > 0 && quad_head<L>(vel_index<L>(a, b));
}

// Raw moments of one quadruple: with u1 = f(a,b) + f(-a,-b), u2 = f(a,b) - f(-a,-b),
// u3 = f(a,-b) + f(-a,b), u4 = f(a,-b) - f(-a,b), a moment M_kl gains a^k b^l times
// u1 + u3 (k, l even), u1 - u3 (both odd), u2 - u4 (k even, l odd) or u2 + u4 (k odd, l even).
template <class L, int I, class CT>
__device__ __forceinline__ void mrt_accumulate_quad(CT* M, bool* set, CT fpp, CT fpm, CT fmp, CT fmm) {
  const CT u1 = ladd(fpp, fmm), u2 = lsub(fpp, fmm), u3 = ladd(fpm, fmp), u4 = lsub(fpm, fmp);
  const CT ee = ladd(u1, u3), oo = lsub(u1, u3), eo = lsub(u2, u4), oe = ladd(u2, u4);
  static_for<0, mom_count(L::HN)>([&](auto K) {
    constexpr int k = decltype(K)::value, ka = mom_a(k), kb = mom_b(k);
    constexpr int coef = ipow(L::cx(I), ka) * ipow(L::cy(I), kb);
    const CT& e = (ka & 1) ? ((kb & 1) ? oo : oe) : ((kb & 1) ? eo : ee);
    acc_add<coef>(M[k], set[k], e);
  });
}

// Regularised MRT collision on one node (mrt.jl:56-118), written with raw moments: the
// Hermite coefficients a_f^(n) = Σ f_i H_n(c_i) of orders 2..N are formed from the raw
// moments M_ab, relaxed towards a_eq^(n) = ρ u^{⊗n}, and the populations are rebuilt as
// w_i (ρ + cs ρ u·c_i + Σ_n cs^n / n! a_coll^(n) : H_n(c_i)), expanded in monomials of c_i.
// DEV: v holds g = f - w and receives g_out = f_out - w.  The weights' own Hermite moments
// of orders 1..N vanish (the quadrature symmetry the reference tests, test/quadrature.jl:1-19),
// so the coefficients of f equal those formed from g, with ρ - 1 in place of ρ where M_00 enters.
// Velocities off the axes are taken four at a time, {(±a, ±b)}, through their parity
// combinations (one term per moment for the four), axis velocities in opposite pairs.
// `pop(std::integral_constant<int, i>)` supplies population i; `out(i, value)` receives it.
template <class L, bool DEV, class CT, class Pop, class Out>
__device__ __forceinline__ void mrt_node(const StepParams<CT>& p, CT sFx, CT sFy, bool has_force, Pop&& pop,
                                         Out&& out) {
  constexpr int NM = mom_count(L::HN);
  CT M[15];
  bool ms[15];
  static_for<0, 15>([&](auto K) { ms[decltype(K)::value] = false; });
  static_for<0, L::Q>([&](auto I) {
    constexpr int i = decltype(I)::value, o = L::opp(i);
    if constexpr (o == i) {
      acc_add<1>(M[0], ms[0], pop(I));
    } else if constexpr (quad_head<L>(i)) {
      constexpr int ipm = vel_index<L>(L::cx(i), -L::cy(i)), imp = vel_index<L>(-L::cx(i), L::cy(i));
      mrt_accumulate_quad<L, i>(M, ms, pop(I), pop(std::integral_constant<int, ipm>{}),
                                pop(std::integral_constant<int, imp>{}), pop(std::integral_constant<int, o>{}));
    } else if constexpr (!in_quad<L>(i) && o > i) {
      const CT a = pop(I), b = pop(std::integral_constant<int, o>{});
      mrt_accumulate_pair<L, i>(M, ms, ladd(a, b), lsub(a, b));
    }
  });
  static_for<0, NM>([&](auto K) {
    constexpr int k = decltype(K)::value;
    if (!ms[k]) M[k] = (CT)0;
  });
  MrtCoeffs<CT> c;
  mrt_coeffs<L, DEV>(p, M, sFx, sFy, has_force, c);
  static_for<0, L::Q>([&](auto I) {
    constexpr int i = decltype(I)::value, o = L::opp(i);
    if constexpr (o == i) {
      out(i, p.w[i] * c.B[0]);
    } else if constexpr (quad_head<L>(i)) {
      // parity sums P_ee, P_eo, P_oe, P_oo of the monomials at (a, b); the four outputs are their
      // signed combinations (first-order terms with w1 in deviation storage)
      constexpr int ipm = vel_index<L>(L::cx(i), -L::cy(i)), imp = vel_index<L>(-L::cx(i), L::cy(i));
      CT P[4];  // ee, eo, oe, oo
      bool ps[4] = {true, false, false, false};
      P[0] = c.B[0];
      static_for<(DEV ? 3 : 1), NM>([&](auto K) {
        constexpr int k = decltype(K)::value, ka = mom_a(k), kb = mom_b(k);
        constexpr int coef = ipow(L::cx(i), ka) * ipow(L::cy(i), kb);
        constexpr int slot = ((ka & 1) ? 2 : 0) + ((kb & 1) ? 1 : 0);
        acc_add<coef>(P[slot], ps[slot], c.B[k]);
      });
      const CT w = p.w[i];
      const CT Tee = w * P[0];
      CT Teo = ps[1] ? w * P[1] : (CT)0, Toe = ps[2] ? w * P[2] : (CT)0;
      const CT Too = ps[3] ? w * P[3] : (CT)0;
      if constexpr (DEV) {
        Teo = ladd(Teo, p.w1[i] * ((CT)L::cy(i) * c.B2p));
        Toe = ladd(Toe, p.w1[i] * ((CT)L::cx(i) * c.B1p));
      }
      const CT v1 = ladd(Tee, Too), v2 = lsub(Tee, Too), v3 = ladd(Teo, Toe), v4 = lsub(Toe, Teo);
      out(i, v1 + v3);
      out(o, v1 - v3);
      out(ipm, v2 + v4);
      out(imp, v2 - v4);
    } else if constexpr (!in_quad<L>(i) && o > i) {
      CT a, b;
      mrt_out_pair<L, DEV, i>(p, c, a, b);
      out(i, a);
      out(o, b);
    }
  });
}

template <class L, bool DEV, class CT>
__device__ __forceinline__ void mrt_collide(const StepParams<CT>& p, CT* v, CT sFx, CT sFy, bool has_force) {
  CT r[L::Q];
  mrt_node<L, DEV>(p, sFx, sFy, has_force, [&](auto I) { return v[decltype(I)::value]; },
                   [&](int i, CT val) { r[i] = val; });
  static_for<0, L::Q>([&](auto I) { v[decltype(I)::value] = r[decltype(I)::value]; });
}

// 1/ρ for the O(u²) terms of the pair form.  FP64: a float reciprocal refined by one
// Newton-Raphson step r (2 - ρ r), relative error ~1e-14, well below what the terms it scales
// (u² ~ 1e-4 of f) need; FP32: the hardware reciprocal; float-float: recip() of lbm_df64.cuh.
__device__ __forceinline__ double pair_recip(double r) {
  // the float approximation is formed from the bits of r (no FP64-pipe conversions): exponent
  // rebiased, significand truncated to 23 bits; densities lie well inside float's exponent range,
  // anything else (≤ 0, tiny, huge, NaN) takes the full division
  const long long b = __double_as_longlong(r);
  const int e = (int)((b >> 52) & 0x7FF);
  if (b > 0 && e > 1023 - 120 && e < 1023 + 120) {
    const float rf = __int_as_float(((e - 1023 + 127) << 23) | (int)((b >> 29) & 0x7FFFFF));
    const int rb = __float_as_int(__frcp_rn(rf));
    const double r0 =
        __longlong_as_double(((long long)(((rb >> 23) & 0xFF) - 127 + 1023) << 52) | ((long long)(rb & 0x7FFFFF) << 29));
    return fma(r0, fma(-r, r0, 1.0), r0);
  }
  return 1.0 / r;
}
__device__ __forceinline__ float pair_recip(float r) { return __frcp_rn(r); }
__device__ __forceinline__ dd pair_recip(dd r) { return recip(r); }

__device__ __forceinline__ bool nonzero_bits(double v) { return __double_as_longlong(v) != 0; }
__device__ __forceinline__ bool nonzero_bits(float v) { return __float_as_int(v) != 0; }
__device__ __forceinline__ bool nonzero_bits(dd v) { return __float_as_int(v.hi) != 0 || __float_as_int(v.lo) != 0; }

// Velocity class of population i: the set {(±a, ±b), (±b, ±a)}, which shares one weight.
template <class L>
__host__ __device__ constexpr int vclass(int i) {
  const int a = L::cx(i) < 0 ? -L::cx(i) : L::cx(i), b = L::cy(i) < 0 ? -L::cy(i) : L::cy(i);
  return a < b ? a * 4 + b : b * 4 + a;
}
template <class L>
__host__ __device__ constexpr bool class_first(int i) {
  for (int j = 0; j < i; ++j)
    if (vclass<L>(j) == vclass<L>(i)) return false;
  return true;
}

// A node's collision split over PARTS warps (the block-resident batched kernel, lbm_resident.cuh):
// every part computes the node-wide quantities, and part PART computes and owns the outputs of the
// opposite pairs whose ordinal (pairs counted in population order) is PART modulo PARTS, the rest
// population going to part 0.  Each output is formed by the same operations whichever part forms
// it, so a split collision gives the bits of the whole one.
template <class L>
__host__ __device__ constexpr int pair_ordinal(int i) {  // i: the lower index of an opposite pair
  int k = 0;
  for (int j = 0; j < i; ++j)
    if (L::opp(j) > j) ++k;
  return k;
}
template <class L, int PARTS, int PART>
__host__ __device__ constexpr bool owns_pop(int i) {
  if (PARTS == 1) return true;
  const int o = L::opp(i);
  if (o == i) return PART == 0;
  return pair_ordinal<L>(o < i ? o : i) % PARTS == PART;
}
template <class L, int PARTS, int PART>
__host__ __device__ constexpr bool class_needed(int cls) {  // a population of class cls is PART's output
  for (int j = 0; j < L::Q; ++j)
    if (vclass<L>(j) == cls && owns_pop<L, PARTS, PART>(j)) return true;
  return false;
}

// SRT / TRT in "pair form" (all storages).  Opposite populations enter only through their
// sum s and difference d, which give both the moments (δρ = Σ s, j = Σ c d) and the TRT
// symmetric / antisymmetric parts; the equilibrium is built from j' = ρ(u + τF) directly, with
// X = c_i·j', J² = |j'|², c = 1/c_s²:
//   feq_i = S + A,  feq_opp(i) = S - A,
//   S = w δρ + w (c²X² - cJ²) / (2ρ) [+ w (c⁴X⁴ - 6c³J²X² + 3c²J⁴) / (24ρ³)  fourth order]
//   A = w1 X                          [+ w c X (c²X² - 3cJ²) / (6ρ²)          third order]
// (the truncations of velocity_distribution_function/*.jl written in j'), and the update is
// f'_i = Ys + Ya, f'_opp = Ys - Ya with Ys = (1 - ω_s) s/2 + ω_s S, Ya = (1 - ω_a) d/2 + ω_a A
// (srt.jl:18-62 and trt.jl:42-97 rewritten; SRT is ω_s = ω_a).  ω_s S and ω_a A are
// polynomials in X whose coefficients depend on the node and the weight only, so they are
// formed once per velocity class: ω_s S = b0 + X² (b2 + X² b4), ω_a A = X (ω_a w1 + a3 (c²X² - 3cJ²)).
// FP32 keeps ω_a (w1 X) with the FP32-exact w1, so the equilibrium's momentum stays exact.
// CT is the type of the node values and PT that of the parameters: the same type, or packed FP32
// pairs (pf2, two nodes) with FP32 parameters.
template <class L, bool DEV, int PARTS = 1, int PART = 0, class CT, class PT>
__device__ __forceinline__ void collide_pairs(const StepParams<PT>& p, CT* v, CT sFx, CT sFy, bool has_force) {
  constexpr bool F32 = std::is_same<CT, float>::value || std::is_same<CT, pf2>::value;
  CT sp[L::Q], dp[L::Q];
  CT drho, jx, jy;
  bool sr = false, sx = false, sy = false;
  static_for<0, L::Q>([&](auto I) {
    constexpr int i = decltype(I)::value, o = L::opp(i);
    if constexpr (o == i) {
      acc_add<1>(drho, sr, v[i]);
    } else if constexpr (o > i) {
      sp[i] = ladd(v[i], v[o]);
      dp[i] = lsub(v[i], v[o]);
      acc_add<1>(drho, sr, sp[i]);
    }
  });
  static_for<0, L::Q>([&](auto I) {
    constexpr int i = decltype(I)::value, o = L::opp(i);
    if constexpr (o > i) {
      acc_add<L::cx(i)>(jx, sx, dp[i]);
      acc_add<L::cy(i)>(jy, sy, dp[i]);
    }
  });
  // FP64 storage holds f, so `drho` is ρ itself and w·drho below is w ρ; deviation storage
  // holds g = f - w, so it is ρ - 1 and w·drho is the deviation w (ρ - 1) of the rest state
  const CT rho = DEV ? ladd((CT)1, drho) : drho;
  const CT inv = pair_recip(rho);
  if (has_force) {  // j' = ρ (u + τ F); a zero component adds nothing (tested on its bits, not on the FP64 pipe)
    if (nonzero_bits(sFx)) jx = add_prod(jx, rho, sFx);
    if (nonzero_bits(sFy)) jy = add_prod(jy, rho, sFy);
  }
  // node-wide, weight-free factors of b0, b2, b4 and a3
  CT D0 = drho, D2 = 0, D4 = 0, J2 = 0, c3 = 0, cs3J2 = 0, csq = 0;
  if constexpr (L::EQ >= 2) {
    J2 = prod_add(jx, jx, jy * jy);
    D0 = sub_prod(drho, p.hcs * J2, inv);
    D2 = p.hcs2 * inv;
  }
  if constexpr (L::EQ >= 3) {
    c3 = p.cs * (CT)(1.0 / 6.0) * (inv * inv);  // c / (6 ρ²)
    cs3J2 = (CT)3 * p.cs * J2;                  // 3 c J²
    csq = p.cs * p.cs;
  }
  if constexpr (L::EQ >= 4) {
    const CT c4 = (CT)(1.0 / 24.0) * (inv * inv) * inv;  // 1 / (24 ρ³)
    D0 = add_prod(D0, ((CT)3 * csq) * (J2 * J2), c4);
    D2 = sub_prod(D2, ((CT)6 * (csq * p.cs)) * J2, c4);
    D4 = (csq * csq) * c4;
  }
  CT b0[16], b2[16], b4[16], a3[16];
  static_for<0, L::Q>([&](auto I) {
    constexpr int i = decltype(I)::value;
    if constexpr (class_first<L>(i) && class_needed<L, PARTS, PART>(vclass<L>(i))) {
      constexpr int k = vclass<L>(i);
      b0[k] = p.pws[i] * D0;
      if constexpr (L::EQ >= 2) b2[k] = p.pws[i] * D2;
      if constexpr (L::EQ >= 4) b4[k] = p.pws[i] * D4;
      if constexpr (L::EQ >= 3) a3[k] = (F32 ? p.w[i] : p.pwa[i]) * c3;
    }
  });
  static_for<0, L::Q>([&](auto I) {
    constexpr int i = decltype(I)::value, o = L::opp(i), k = vclass<L>(i);
    if constexpr (o == i && PART == 0) {
      v[i] = prod_add_out(p.pa_s2, v[i], b0[k]);
    } else if constexpr (o > i && owns_pop<L, PARTS, PART>(i)) {
      // X = c_i·j': a unit coefficient enters first, so that an integer multiple (|c| = 2, 3) is
      // added by an explicit FMA rather than a product the compiler may or may not fuse
      CT X;
      bool xs = false;
      constexpr int ax = L::cx(i) < 0 ? -L::cx(i) : L::cx(i), ay = L::cy(i) < 0 ? -L::cy(i) : L::cy(i);
      if constexpr (ax > 1 && ay == 1) {
        acc_add<L::cy(i)>(X, xs, jy);
        acc_add<L::cx(i)>(X, xs, jx);
      } else {
        acc_add<L::cx(i)>(X, xs, jx);
        acc_add<L::cy(i)>(X, xs, jy);
      }
      [[maybe_unused]] const CT X2 = X * X;
      CT Se = b0[k];
      if constexpr (L::EQ >= 4) Se = add_prod(Se, X2, add_prod(b2[k], X2, b4[k]));
      else if constexpr (L::EQ >= 2) Se = add_prod(Se, X2, b2[k]);
      CT Ya;
      if constexpr (F32) {
        CT A = p.w1[i] * X;
        if constexpr (L::EQ >= 3) A = add_prod(A, X * prod_sub(csq, X2, cs3J2), a3[k]);
        Ya = prod_add(p.pa_a, dp[i], p.pom_a * A);
      } else {
        CT t = p.pw1a[i];
        if constexpr (L::EQ >= 3) t = add_prod(t, a3[k], prod_sub(csq, X2, cs3J2));
        Ya = prod_add(p.pa_a, dp[i], t * X);
      }
      const CT Ys = prod_add(p.pa_s, sp[i], Se);
      v[i] = Ys + Ya;
      v[o] = Ys - Ya;
    }
  });
}

// Collision of one node in place (v holds f for F64, g = f - w for deviation storage).
//   SRT  srt.jl:18-62    f_out = (1 - 1/τ) f + (1/τ) feq(ρ, u + τF)
//   TRT  trt.jl:42-97    symmetric / antisymmetric parts relaxed with τ_s / τ_a, u + τ_a F
//   MRT  mrt.jl:56-118   regularised projection (mrt_collide)
//   ITER iterative_initialization.jl:41-60   feq = w ρ + nonlinear term
// `time()` gives the physical time of the step (step_time(p), or a batch member's own).
// PARTS / PART split an SRT / TRT collision over warps (see owns_pop); MRT and the iterative
// collision are never split.
template <class L, class S, int COLL, int PARTS = 1, int PART = 0, class CT, class TimeFn>
__device__ __forceinline__ void collide_node(const StepParams<CT>& p, int x, int y, CT* v, TimeFn&& time) {
  static_assert(PARTS == 1 || COLL == LBM_SRT || COLL == LBM_TRT, "only the pair-form collisions split");
  constexpr bool DEV = S::DEV;
  if constexpr (COLL == LBM_ITERATIVE_INIT) {
    CT s = v[0];
#pragma unroll
    for (int i = 1; i < L::Q; ++i) s += v[i];
    const CT rho = DEV ? (CT)1 + s : s;
    const size_t node = (size_t)y * p.nx + x;
#pragma unroll
    for (int i = 0; i < L::Q; ++i) {
      const CT nl = p.nonlinear[plane_off(p, i) + node];
      const CT feq = DEV ? p.w[i] * s + nl : p.w[i] * rho + nl;
      v[i] = p.om_a * v[i] + p.om_b * feq;
    }
  } else {
    CT sFx = 0, sFy = 0;
    const bool has_force = p.force_kind != LBM_FORCE_NONE;
    if (has_force) node_shifted_force(p, x, y, sFx, sFy, time);
    if constexpr (COLL == LBM_MRT) mrt_collide<L, DEV>(p, v, sFx, sFy, has_force);
    else collide_pairs<L, DEV, PARTS, PART>(p, v, sFx, sFy, has_force);
  }
}

// ---------------------------------------------------------------------------------------
// Kernels.  Grid: x blocks of 128 threads along x, one row of y per block row.
// ---------------------------------------------------------------------------------------
constexpr int kBlockX = 128;

// MODE 0: collide only (first step after an upload: f_stream -> f_collision)
// MODE 1: fused pull + boundaries + collide (post-collision -> post-collision)
// MODE 2: pull + boundaries only (post-collision -> f_stream, materialising the observable state)
// The float-float D2Q37 regularised MRT asks for 4 resident blocks: 128 registers without spills
// (left alone the compiler takes 96 and spills), 6.6 against 6.2 GLUPS on the 2048^2 shear wave;
// a bound of 6 blocks (80 registers, 84 bytes spilled) ran at 6.1.
template <class L, class S, int COLL, int MODE>
__global__ void __launch_bounds__(kBlockX, (COLL == LBM_MRT && (S::id == LBM_STORE_DF64_DEV || S::id == LBM_STORE_F32_DEV_SR) && L::Q == 37) ? 4 : 0) step_kernel(StepParams<typename S::C> p,
                                                       const typename S::T* __restrict__ src,
                                                       typename S::T* __restrict__ dst) {
  using CT = typename S::C;
  // FP64-DD MRT: per-thread staging slots, one per population (a float-float pair has the 8 bytes
  // of the double it replaces; no thread reads another's slots, so no barrier): the double <->
  // float-float conversions run in loops instead of being inlined Q times each
  constexpr bool kStage = S::WIDE && COLL == LBM_MRT && MODE != 2;
  __shared__ double stage[kStage ? L::Q : 1][kStage ? kBlockX : 1];
  wait_prior_grid();
  const int x = blockIdx.x * kBlockX + threadIdx.x;
  if (x >= p.nx) return;
  for (int y = blockIdx.y; y < p.ny; y += gridDim.y) {
    const int node = y * p.nx + x;
    if constexpr (COLL == LBM_MRT && MODE != 2) {
      // streaming form: populations feed the raw moments as they arrive and the outputs are
      // rebuilt and stored one by one, so no per-node array of Q populations stays live
      CT sFx = 0, sFy = 0;
      const bool has_force = p.force_kind != LBM_FORCE_NONE;
      if (has_force) node_shifted_force(p, x, y, sFx, sFy, [&] { return step_time(p); });
      auto out = [&](int i, CT val) { store_out<S>(p, dst, i, node, val); };
      if constexpr (kStage) {
        int xw[2 * L::R + 1], yo[2 * L::R + 1];
        bool staged = true;
        if constexpr (MODE == 0) {
          static_for<0, L::Q>([&](auto I) {
            constexpr int i = decltype(I)::value;
            stage[i][threadIdx.x] = src[plane_off(p, i) + node];
          });
        } else {
          pull_offsets<L>(p, x, y, xw, yo);
          staged = !(p.nbc > 0 && (y < L::R || y >= p.ny - L::R || x < L::R || x >= p.nx - L::R));
          if (staged)
            static_for<0, L::Q>([&](auto I) {
              constexpr int i = decltype(I)::value;
              stage[i][threadIdx.x] = src[plane_off(p, i) + yo[L::R + L::cy(i)] + xw[L::R + L::cx(i)]];
            });
        }
        if (staged) {
#pragma unroll 1
          for (int i = 0; i < L::Q; ++i) {
            const CT g = S::from_f(stage[i][threadIdx.x], p.wf[i]);
            stage[i][threadIdx.x] = __hiloint2double(__float_as_int(g.hi), __float_as_int(g.lo));
          }
          mrt_node<L, S::DEV>(p, sFx, sFy, has_force,
                              [&](auto I) {
                                const double b = stage[decltype(I)::value][threadIdx.x];
                                return CT(__int_as_float(__double2hiint(b)), __int_as_float(__double2loint(b)));
                              },
                              [&](int i, CT val) {
                                stage[i][threadIdx.x] = __hiloint2double(__float_as_int(val.hi), __float_as_int(val.lo));
                              });
#pragma unroll 1
          for (int i = 0; i < L::Q; ++i) {
            const double b = stage[i][threadIdx.x];
            dst[plane_off(p, i) + node] =
                S::to_f(CT(__int_as_float(__double2hiint(b)), __int_as_float(__double2loint(b))), p.wf[i]);
          }
        } else {  // nodes within R of a wall: the pull with its boundary rules, conversions inline
          mrt_node<L, S::DEV>(p, sFx, sFy, has_force,
                              [&](auto I) { return pop_streamed<L, S>(p, src, x, y, xw, yo, true, decltype(I)::value); },
                              out);
        }
      } else if constexpr (MODE == 0) {
        mrt_node<L, S::DEV>(p, sFx, sFy, has_force,
                            [&](auto I) {
                              constexpr int i = decltype(I)::value;
                              return load_pop<S>(p, src + plane_off(p, i) + node, i);
                            }, out);
      } else {
        int xw[2 * L::R + 1], yo[2 * L::R + 1];
        pull_offsets<L>(p, x, y, xw, yo);
        const bool near = p.nbc > 0 && (y < L::R || y >= p.ny - L::R || x < L::R || x >= p.nx - L::R);
        if (near) {
          mrt_node<L, S::DEV>(p, sFx, sFy, has_force,
                              [&](auto I) { return pop_streamed<L, S>(p, src, x, y, xw, yo, true, decltype(I)::value); },
                              out);
        } else {
          mrt_node<L, S::DEV>(p, sFx, sFy, has_force, [&](auto I) {
            constexpr int i = decltype(I)::value;
            return load_pop<S>(p, src + plane_off(p, i) + yo[L::R + L::cy(i)] + xw[L::R + L::cx(i)], i);
          }, out);
        }
      }
    } else {
      CT v[L::Q];
      if (MODE == 0) load_local<L, S>(p, src, node, v);
      else load_streamed<L, S>(p, src, x, y, v);
      if (MODE != 2) {
        collide_node<L, S, COLL>(p, x, y, v, [&] { return step_time(p); });
#pragma unroll
        for (int i = 0; i < L::Q; ++i) store_out<S>(p, dst, i, node, v[i]);
      } else {
#pragma unroll
        for (int i = 0; i < L::Q; ++i) store_pop<S>(p, dst + plane_off(p, i) + node, i, v[i]);
      }
    }
  }
}

// Fused step (MODE 1) of SRT / TRT with FP32 or float-float arithmetic, two x-adjacent nodes
// (x0, x0 + 1), x0 even, per thread.  The collision runs on packed FP32 pairs (pf2 / pdd,
// lbm_pf2.cuh), so its arithmetic issues once for both nodes; the populations with c_x = 0 are
// loaded, and all outputs stored, as one aligned two-node access; away from the x edges the
// second node's addresses are the first's plus one element.  Nodes within R of an x edge, or of
// a y edge when boundary conditions are set, are pulled by load_streamed.  Needs nx even.
// Residency: FP16 D2Q4-D2Q9 ten blocks per SM (48 registers), F64DD and FP32-SR seven (72
// registers, a few spilled words; D2Q9 4096^2: F64DD 20.9 against 20.5 GLUPS at six blocks,
// FP32-SR 41.2 against 40.7 at six and 39.2 at the compiler's 94 registers).
template <class L, class S>
__global__ void __launch_bounds__(kBlockX, (S::id == LBM_STORE_F16_DEV && L::Q <= 9) ? 10 : (S::id == LBM_STORE_F64_DD || S::id == LBM_STORE_F32_DEV_SR ? 7 : 0)) step_pair_kernel(StepParams<typename S::C> p,
                                                            const typename S::T* __restrict__ src,
                                                            typename S::T* __restrict__ dst) {
  using T = typename S::T;
  using C = typename S::C;
  using P = typename Packed<C>::type;
  // FP64-DD: per-thread staging slots of the Q population pairs (16 B each; no thread reads
  // another's, so no barrier), which let the double <-> float-float conversions run in loops
  __shared__ double2 wide_stage[S::WIDE ? L::Q : 1][S::WIDE ? kBlockX : 1];
  wait_prior_grid();
  const int x0 = 2 * (int)(blockIdx.x * kBlockX + threadIdx.x);
  if (x0 >= p.nx) return;
  const bool x_inner = x0 >= L::R && x0 + 1 + L::R < p.nx;
  const bool has_force = p.force_kind != LBM_FORCE_NONE;
  for (int y = blockIdx.y; y < p.ny; y += gridDim.y) {
    const int node = y * p.nx + x0;
    P v[L::Q];
    if (x_inner && !(p.nbc > 0 && (y < L::R || y >= p.ny - L::R))) {
      int yo[2 * L::R + 1];
#pragma unroll
      for (int k = 0; k < 2 * L::R + 1; ++k) {
        int ys = y - p.dym[k - L::R + 3];
        ys += (ys < 0) ? p.ny : 0;
        yo[k] = ys * p.nx;
      }
      if constexpr (S::WIDE) {
        // the raw doubles of both nodes go to this thread's staging slots (all loads in flight at
        // once), one loop converts them in place: one copy of the split code instead of 2 Q
        static_for<0, L::Q>([&](auto I) {
          constexpr int i = decltype(I)::value;
          const T* a = src + plane_off(p, i) + (yo[L::R + L::cy(i)] + x0 - L::cx(i));
          wide_stage[i][threadIdx.x] = make_double2(a[0], a[1]);
        });
#pragma unroll 1
        for (int i = 0; i < L::Q; ++i) {
          const double2 f = wide_stage[i][threadIdx.x];
          const pdd g = pack2(S::from_f(f.x, p.wf[i]), S::from_f(f.y, p.wf[i]));
          wide_stage[i][threadIdx.x] = make_double2(__longlong_as_double((long long)g.hi.r),
                                                    __longlong_as_double((long long)g.lo.r));
        }
        static_for<0, L::Q>([&](auto I) {
          constexpr int i = decltype(I)::value;
          const double2 g = wide_stage[i][threadIdx.x];
          v[i].hi.r = (unsigned long long)__double_as_longlong(g.x);
          v[i].lo.r = (unsigned long long)__double_as_longlong(g.y);
        });
      } else {
        static_for<0, L::Q>([&](auto I) {
          constexpr int i = decltype(I)::value;
          const T* a = src + plane_off(p, i) + (yo[L::R + L::cy(i)] + x0 - L::cx(i));
          if constexpr (L::cx(i) == 0) v[i] = S::ld2(a);
          else v[i] = pack2(S::ld(a), S::ld(a + 1));
        });
      }
    } else {
      C a[L::Q], b[L::Q];
      load_streamed<L, S>(p, src, x0, y, a);
      load_streamed<L, S>(p, src, x0 + 1, y, b);
#pragma unroll
      for (int i = 0; i < L::Q; ++i) v[i] = pack2(a[i], b[i]);
    }
    P sFx = 0, sFy = 0;
    if (has_force) {
      C ax, ay, bx, by;
      auto time = [&] { return step_time(p); };
      node_shifted_force(p, x0, y, ax, ay, time);
      node_shifted_force(p, x0 + 1, y, bx, by, time);
      sFx = pack2(ax, bx);
      sFy = pack2(ay, by);
    }
    collide_pairs<L, S::DEV>(p, v, sFx, sFy, has_force);
#pragma unroll
    for (int i = 0; i < L::Q; ++i) {
      if constexpr (S::SR) {  // both lanes stochastically rounded, stored as one two-node access
        const unsigned step = step_counter(p);
        const float a = round_stochastic(v[i].hi.lo(), v[i].lo.lo(), sr_bits(node, i, step));
        const float b = round_stochastic(v[i].hi.hi(), v[i].lo.hi(), sr_bits(node + 1, i, step));
        *reinterpret_cast<unsigned long long*>(dst + plane_off(p, i) + node) = pf2(a, b).r;
      } else if constexpr (S::WIDE) {  // staged: one loop below forms and stores the doubles
        wide_stage[i][threadIdx.x] = make_double2(__longlong_as_double((long long)v[i].hi.r),
                                                  __longlong_as_double((long long)v[i].lo.r));
      } else {
        S::st2(dst + plane_off(p, i) + node, v[i]);
      }
    }
    if constexpr (S::WIDE) {  // both lanes as one aligned 16-byte store per population
#pragma unroll 1
      for (int i = 0; i < L::Q; ++i) {
        const double2 g = wide_stage[i][threadIdx.x];
        pdd vi;
        vi.hi.r = (unsigned long long)__double_as_longlong(g.x);
        vi.lo.r = (unsigned long long)__double_as_longlong(g.y);
        *reinterpret_cast<double2*>(dst + plane_off(p, i) + node) =
            make_double2(S::to_f(dd(vi.hi.lo(), vi.lo.lo()), p.wf[i]), S::to_f(dd(vi.hi.hi(), vi.lo.hi()), p.wf[i]));
      }
    }
  }
}

}  // namespace lbm
