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

template <class L, class S>
struct Node {
  using C = typename S::C;
  C f[L::Q];
};

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
    f[i] = S::ld(src + (size_t)i * p.n + idx);
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
          if (hit) f[i] = S::ld(src + (size_t)o * p.n + node);
        }
      } else {  // MovingWall{North}: whole top wall, ignores xs / ys
#pragma unroll
        for (int i = 0; i < L::Q; ++i) {
          const int o = L::opp(i);
          if (y1 + L::cy(o) > p.ny) f[i] = S::ld(src + (size_t)o * p.n + node) + (typename S::C)bc.add[i];
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
  typename S::C v = S::ld(src + (size_t)i * p.n + yo[L::R + L::cy(i)] + xw[L::R + L::cx(i)]);
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
        if (hit) v = S::ld(src + (size_t)o * p.n + node);
      } else if (y1 + L::cy(o) > p.ny) {
        v = S::ld(src + (size_t)o * p.n + node) + (typename S::C)bc.add[i];
      }
    }
  }
  return v;
}

template <class L, class S, class CT>
__device__ __forceinline__ void load_local(const StepParams<CT>& p, const typename S::T* __restrict__ src,
                                           int node, typename S::C* f) {
#pragma unroll
  for (int i = 0; i < L::Q; ++i) f[i] = S::ld(src + (size_t)i * p.n + node);
}

// Lattice force at node (x, y), lattice_force(problem, x, y, t) (problems.jl:103-104).
template <class CT>
__device__ __forceinline__ void node_force(const StepParams<CT>& p, int x, int y, CT& Fx, CT& Fy) {
  if (p.force_kind == LBM_FORCE_CONSTANT) {
    Fx = p.F[0];
    Fy = p.F[1];
  } else if (p.force_kind == LBM_FORCE_FIELD) {
    const size_t k = (size_t)y * p.nx + x;
    Fx = (CT)__ldg(p.Ffield + k);
    Fy = (CT)__ldg(p.Ffield + p.n + k);
  } else if (p.force_kind == LBM_FORCE_SHEAR) {
    const double X = __ldg(p.xr + x), Y = __ldg(p.yr + y);
    Fx = (CT)(p.shear[0] * cos(p.shear[1] * Y - p.shear[2] * p.time));
    Fy = (CT)(p.shear[3] * cos(p.shear[4] * X - p.shear[5] * p.time));
  } else {
    Fx = 0;
    Fy = 0;
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

// Regularised MRT collision on one node (mrt.jl:135-197), written with raw moments: the
// Hermite coefficients a_f^(n) = Σ f_i H_n(c_i) of orders 2..N are formed from the raw
// moments M_ab, relaxed towards a_eq^(n) = ρ u^{⊗n}, and the populations are rebuilt as
// w_i (ρ + cs ρ u·c_i + Σ_n cs^n / n! a_coll^(n) : H_n(c_i)), expanded in monomials of c_i.
// DEV: v holds g = f - w and receives g_out = f_out - w.  The weights' own Hermite moments
// of orders 1..N vanish (the quadrature symmetry the reference tests, test/quadrature.jl:1-19),
// so the coefficients of f equal those formed from g, with ρ - 1 in place of ρ where M_00 enters.
template <class CT>
struct MrtCoeffs {
  CT B[15];      // coefficients of the monomials c_x^a c_y^b of f_out / w
  CT B1p, B2p;   // deviation storage: first-order coefficients per w1 = c w
};

template <class L, class CT>
__device__ __forceinline__ void mrt_accumulate(CT* M, int i, CT v) {
  constexpr int NM = mom_count(L::HN);
#pragma unroll
  for (int k = 0; k < NM; ++k) {
    const int coef = ipow(L::cx(i), mom_a(k)) * ipow(L::cy(i), mom_b(k));
    if (coef == 1) M[k] += v;
    else if (coef == -1) M[k] -= v;
    else if (coef != 0) M[k] += (CT)coef * v;
  }
}

// Pair form of mrt_accumulate: opposite populations i, opp(i) enter through s = f_i + f_opp and
// d = f_i - f_opp, since c_opp = -c_i makes each monomial of odd degree flip sign.
template <class L, class CT>
__device__ __forceinline__ void mrt_accumulate_pair(CT* M, int i, CT s, CT d) {
  constexpr int NM = mom_count(L::HN);
#pragma unroll
  for (int k = 0; k < NM; ++k) {
    const int coef = ipow(L::cx(i), mom_a(k)) * ipow(L::cy(i), mom_b(k));
    const CT v = ((mom_a(k) + mom_b(k)) & 1) ? d : s;
    if (coef == 1) M[k] += v;
    else if (coef == -1) M[k] -= v;
    else if (coef != 0) M[k] += (CT)coef * v;
  }
}

// Pair form of mrt_out: the even- and odd-degree parts E, O of population i give
// f_i = w (E + O) and f_opp = w (E - O).
template <class L, bool DEV, class CT>
__device__ __forceinline__ void mrt_out_pair(const StepParams<CT>& p, const MrtCoeffs<CT>& c, int i, CT& out_i,
                                             CT& out_o) {
  constexpr int NM = mom_count(L::HN);
  CT E = c.B[0], O = 0;
#pragma unroll
  for (int k = DEV ? 3 : 1; k < NM; ++k) {
    const int coef = ipow(L::cx(i), mom_a(k)) * ipow(L::cy(i), mom_b(k));
    CT& acc = ((mom_a(k) + mom_b(k)) & 1) ? O : E;
    if (coef == 1) acc += c.B[k];
    else if (coef == -1) acc -= c.B[k];
    else if (coef != 0) acc += (CT)coef * c.B[k];
  }
  CT we = p.w[i] * E, wo = p.w[i] * O;
  if constexpr (DEV) {
    CT s1 = 0;
    if (L::cx(i) != 0) s1 += (CT)L::cx(i) * c.B1p;
    if (L::cy(i) != 0) s1 += (CT)L::cy(i) * c.B2p;
    wo += p.w1[i] * s1;
  }
  out_i = we + wo;
  out_o = we - wo;
}

// Relaxation of the Hermite coefficients from the raw moments M (see mrt_collide).
template <class L, bool DEV, class CT>
__device__ __forceinline__ void mrt_coeffs(const StepParams<CT>& p, const CT* M, CT Fx, CT Fy, bool has_force,
                                           MrtCoeffs<CT>& c) {
  const CT rho = DEV ? (CT)1 + M[0] : M[0];
  const CT inv_rho = (CT)1 / rho;
  CT ux = M[1] * inv_rho, uy = M[2] * inv_rho;
  if (has_force) {
    ux += p.shift * Fx;
    uy += p.shift * Fy;
  }
  const CT cs = p.cs, ics = (CT)1 / cs;  // ics = c_s^2
  CT* B = c.B;
#pragma unroll
  for (int k = 0; k < 15; ++k) B[k] = 0;
  B[0] = M[0];  // ρ, or ρ - 1 in deviation form
  B[1] = cs * rho * ux;
  B[2] = cs * rho * uy;
  c.B1p = rho * ux;
  c.B2p = rho * uy;
  if constexpr (L::HN >= 2) {
    const CT a = p.mrt_a[1], b = p.mrt_b[1];
    const CT Axx = a * (M[3] - ics * M[0]) + b * (rho * ux * ux);
    const CT Axy = a * M[4] + b * (rho * ux * uy);
    const CT Ayy = a * (M[5] - ics * M[0]) + b * (rho * uy * uy);
    const CT c2 = cs * cs * (CT)0.5;
    B[3] += c2 * Axx;
    B[4] += c2 * (CT)2 * Axy;
    B[5] += c2 * Ayy;
    B[0] -= c2 * ics * (Axx + Ayy);
  }
  if constexpr (L::HN >= 3) {
    const CT a = p.mrt_a[2], b = p.mrt_b[2];
    const CT Axxx = a * (M[6] - (CT)3 * ics * M[1]) + b * (rho * ux * ux * ux);
    const CT Axxy = a * (M[7] - ics * M[2]) + b * (rho * ux * ux * uy);
    const CT Axyy = a * (M[8] - ics * M[1]) + b * (rho * ux * uy * uy);
    const CT Ayyy = a * (M[9] - (CT)3 * ics * M[2]) + b * (rho * uy * uy * uy);
    const CT c3 = cs * cs * cs * (CT)(1.0 / 6.0);
    B[6] += c3 * Axxx;
    B[7] += c3 * (CT)3 * Axxy;
    B[8] += c3 * (CT)3 * Axyy;
    B[9] += c3 * Ayyy;
    B[1] -= c3 * (CT)3 * ics * (Axxx + Axyy);
    B[2] -= c3 * (CT)3 * ics * (Axxy + Ayyy);
    c.B1p -= c3 * (CT)3 * ics * ics * (Axxx + Axyy);
    c.B2p -= c3 * (CT)3 * ics * ics * (Axxy + Ayyy);
  }
  if constexpr (L::HN >= 4) {
    const CT a = p.mrt_a[3], b = p.mrt_b[3];
    const CT ics2 = ics * ics;
    const CT Axxxx = a * (M[10] - (CT)6 * ics * M[3] + (CT)3 * ics2 * M[0]) + b * (rho * ux * ux * ux * ux);
    const CT Axxxy = a * (M[11] - (CT)3 * ics * M[4]) + b * (rho * ux * ux * ux * uy);
    const CT Axxyy = a * (M[12] - ics * (M[3] + M[5]) + ics2 * M[0]) + b * (rho * ux * ux * uy * uy);
    const CT Axyyy = a * (M[13] - (CT)3 * ics * M[4]) + b * (rho * ux * uy * uy * uy);
    const CT Ayyyy = a * (M[14] - (CT)6 * ics * M[5] + (CT)3 * ics2 * M[0]) + b * (rho * uy * uy * uy * uy);
    const CT c4 = cs * cs * cs * cs * (CT)(1.0 / 24.0);
    B[10] += c4 * Axxxx;
    B[11] += c4 * (CT)4 * Axxxy;
    B[12] += c4 * (CT)6 * Axxyy;
    B[13] += c4 * (CT)4 * Axyyy;
    B[14] += c4 * Ayyyy;
    B[3] -= c4 * ics * (CT)6 * (Axxxx + Axxyy);
    B[4] -= c4 * ics * (CT)12 * (Axxxy + Axyyy);
    B[5] -= c4 * ics * (CT)6 * (Axxyy + Ayyyy);
    B[0] += c4 * ics2 * ((CT)3 * Axxxx + (CT)6 * Axxyy + (CT)3 * Ayyyy);
  }
}

// Post-collision population i rebuilt from the coefficients.  Deviation storage: the first-order
// monomials carry w1_i / c instead of w_i (see collide_pairs).
template <class L, bool DEV, class CT>
__device__ __forceinline__ CT mrt_out(const StepParams<CT>& p, const MrtCoeffs<CT>& c, int i) {
  constexpr int NM = mom_count(L::HN);
  CT s = c.B[0];
#pragma unroll
  for (int k = DEV ? 3 : 1; k < NM; ++k) {
    const int coef = ipow(L::cx(i), mom_a(k)) * ipow(L::cy(i), mom_b(k));
    if (coef == 1) s += c.B[k];
    else if (coef == -1) s -= c.B[k];
    else if (coef != 0) s += (CT)coef * c.B[k];
  }
  if constexpr (DEV) {
    CT s1 = 0;
    if (L::cx(i) != 0) s1 += (CT)L::cx(i) * c.B1p;
    if (L::cy(i) != 0) s1 += (CT)L::cy(i) * c.B2p;
    return p.w[i] * s + p.w1[i] * s1;
  } else {
    return p.w[i] * s;
  }
}

// Regularised MRT collision on one node (mrt.jl:135-197), written with raw moments: the
// Hermite coefficients a_f^(n) = Σ f_i H_n(c_i) of orders 2..N are formed from the raw
// moments M_ab, relaxed towards a_eq^(n) = ρ u^{⊗n}, and the populations are rebuilt as
// w_i (ρ + cs ρ u·c_i + Σ_n cs^n / n! a_coll^(n) : H_n(c_i)), expanded in monomials of c_i.
// DEV: v holds g = f - w and receives g_out = f_out - w.  The weights' own Hermite moments
// of orders 1..N vanish (the quadrature symmetry the reference tests, test/quadrature.jl:1-19),
// so the coefficients of f equal those formed from g, with ρ - 1 in place of ρ where M_00 enters.
template <class L, bool DEV, class CT>
__device__ __forceinline__ void mrt_collide(const StepParams<CT>& p, CT* v, CT Fx, CT Fy, bool has_force) {
  CT M[15];
#pragma unroll
  for (int k = 0; k < 15; ++k) M[k] = 0;
#pragma unroll
  for (int i = 0; i < L::Q; ++i) mrt_accumulate<L>(M, i, v[i]);
  MrtCoeffs<CT> c;
  mrt_coeffs<L, DEV>(p, M, Fx, Fy, has_force, c);
#pragma unroll
  for (int i = 0; i < L::Q; ++i) v[i] = mrt_out<L, DEV>(p, c, i);
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
// (srt.jl:18-62 and trt.jl:42-97 rewritten; SRT is ω_s = ω_a).
template <class L, bool DEV, class CT>
__device__ __forceinline__ void collide_pairs(const StepParams<CT>& p, CT* v, CT Fx, CT Fy, bool has_force) {
  CT sp[L::Q], dp[L::Q];
  CT drho = 0;
#pragma unroll
  for (int i = 0; i < L::Q; ++i) {
    const int o = L::opp(i);
    if (o == i) {
      drho += v[i];
    } else if (o > i) {
      sp[i] = v[i] + v[o];
      dp[i] = v[i] - v[o];
      drho += sp[i];
    }
  }
  CT jx = 0, jy = 0;
#pragma unroll
  for (int i = 0; i < L::Q; ++i) {
    const int o = L::opp(i);
    if (o <= i) continue;
    if (L::cx(i) == 1) jx += dp[i];
    else if (L::cx(i) == -1) jx -= dp[i];
    else if (L::cx(i) != 0) jx += (CT)L::cx(i) * dp[i];
    if (L::cy(i) == 1) jy += dp[i];
    else if (L::cy(i) == -1) jy -= dp[i];
    else if (L::cy(i) != 0) jy += (CT)L::cy(i) * dp[i];
  }
  // FP64 storage holds f, so `drho` is ρ itself and w·drho below is w ρ; deviation storage
  // holds g = f - w, so it is ρ - 1 and w·drho is the deviation w (ρ - 1) of the rest state
  const CT rho = DEV ? (CT)1 + drho : drho;
  const CT inv = (CT)1 / rho;
  if (has_force) {  // j' = ρ (u + τ F)
    const CT rs = rho * p.shift;
    jx += rs * Fx;
    jy += rs * Fy;
  }
  CT q2 = 0, J2 = 0, inv2 = 0, c3 = 0, c4 = 0, q4 = 0, cs3J2 = 0;
  if constexpr (L::EQ >= 2) {
    J2 = jx * jx + jy * jy;
    q2 = (p.hcs * J2) * inv;
  }
  if constexpr (L::EQ >= 3) {
    inv2 = inv * inv;
    c3 = p.cs * (CT)(1.0 / 6.0) * inv2;  // c / (6 ρ²)
    cs3J2 = (CT)3 * p.cs * J2;           // 3 c J²
  }
  if constexpr (L::EQ >= 4) {
    c4 = (CT)(1.0 / 24.0) * inv2 * inv;  // 1 / (24 ρ³)
    q4 = (CT)3 * (p.cs * p.cs) * (J2 * J2);
  }
#pragma unroll
  for (int i = 0; i < L::Q; ++i) {
    const int o = L::opp(i);
    if (o == i) {
      CT S = p.w[i] * drho;
      if constexpr (L::EQ >= 2) S -= p.w[i] * q2;
      if constexpr (L::EQ >= 4) S += p.w[i] * (q4 * c4);
      v[i] = ((CT)2 * p.pa_s) * v[i] + p.pom_s * S;
    } else if (o > i) {
      CT X = 0;
      if (L::cx(i) == 1) X += jx;
      else if (L::cx(i) == -1) X -= jx;
      else if (L::cx(i) != 0) X += (CT)L::cx(i) * jx;
      if (L::cy(i) == 1) X += jy;
      else if (L::cy(i) == -1) X -= jy;
      else if (L::cy(i) != 0) X += (CT)L::cy(i) * jy;
      CT S = p.w[i] * drho;
      const CT X2 = X * X;
      if constexpr (L::EQ >= 2) S += p.w[i] * ((p.hcs2 * X2) * inv - q2);
      if constexpr (L::EQ >= 4) {
        const CT cs2 = p.cs * p.cs;
        S += p.w[i] * (((cs2 * cs2) * (X2 * X2) - ((CT)6 * (cs2 * p.cs)) * (J2 * X2) + q4) * c4);
      }
      CT A = p.w1[i] * X;
      if constexpr (L::EQ >= 3) A += p.w[i] * ((X * ((p.cs * p.cs) * X2 - cs3J2)) * c3);
      const CT Ys = p.pa_s * sp[i] + p.pom_s * S;
      const CT Ya = p.pa_a * dp[i] + p.pom_a * A;
      v[i] = Ys + Ya;
      v[o] = Ys - Ya;
    }
  }
}

// Collision of one node in place (v holds f for F64, g = f - w for deviation storage).
//   SRT  srt.jl:18-62    f_out = (1 - 1/τ) f + (1/τ) feq(ρ, u + τF)
//   TRT  trt.jl:42-97    symmetric / antisymmetric parts relaxed with τ_s / τ_a, u + τ_a F
//   MRT  mrt.jl:56-118   regularised projection (mrt_collide)
//   ITER iterative_initialization.jl:41-60   feq = w ρ + nonlinear term
template <class L, class S, int COLL, class CT>
__device__ __forceinline__ void collide_node(const StepParams<CT>& p, int x, int y, CT* v) {
  constexpr bool DEV = S::DEV;
  CT Fx = 0, Fy = 0;
  const bool has_force = p.force_kind != LBM_FORCE_NONE;
  if (COLL != LBM_ITERATIVE_INIT && has_force) node_force(p, x, y, Fx, Fy);
  if constexpr (COLL == LBM_MRT) {
    mrt_collide<L, DEV>(p, v, Fx, Fy, has_force);
    return;
  } else if constexpr (COLL == LBM_SRT || COLL == LBM_TRT) {
    collide_pairs<L, DEV>(p, v, Fx, Fy, has_force);
    return;
  } else {
    CT s = v[0];
#pragma unroll
    for (int i = 1; i < L::Q; ++i) s += v[i];
    const CT rho = DEV ? (CT)1 + s : s;
    const CT drho = DEV ? s : s;  // only used in deviation form
    if constexpr (COLL == LBM_ITERATIVE_INIT) {
      const size_t node = (size_t)y * p.nx + x;
#pragma unroll
      for (int i = 0; i < L::Q; ++i) {
        const CT nl = p.nonlinear[(size_t)i * p.n + node];
        const CT feq = DEV ? p.w[i] * drho + nl : p.w[i] * rho + nl;
        v[i] = p.om_a * v[i] + p.om_b * feq;
      }
      return;
    } else {
      CT jx = 0, jy = 0;
#pragma unroll
      for (int i = 0; i < L::Q; ++i) {
        if (L::cx(i) == 1) jx += v[i];
        else if (L::cx(i) == -1) jx -= v[i];
        else if (L::cx(i) != 0) jx += (CT)L::cx(i) * v[i];
        if (L::cy(i) == 1) jy += v[i];
        else if (L::cy(i) == -1) jy -= v[i];
        else if (L::cy(i) != 0) jy += (CT)L::cy(i) * v[i];
      }
      const CT inv_rho = (CT)1 / rho;
      CT ux = jx * inv_rho, uy = jy * inv_rho;
      if (has_force) {
        ux += p.shift * Fx;
        uy += p.shift * Fy;
      }
      const CT usq = ux * ux + uy * uy;
      CT feq[L::Q];
#pragma unroll
      for (int i = 0; i < L::Q; ++i) {
        CT cu = 0;
        if (L::cx(i) == 1) cu += ux;
        else if (L::cx(i) == -1) cu -= ux;
        else if (L::cx(i) != 0) cu += (CT)L::cx(i) * ux;
        if (L::cy(i) == 1) cu += uy;
        else if (L::cy(i) == -1) cu -= uy;
        else if (L::cy(i) != 0) cu += (CT)L::cy(i) * uy;
        // F64: feq = ρ w (1 + P) as the reference forms it.  Deviation storage: geq = feq - w =
        // w δρ + ρ (w1 c·u + w P_{>=2}), with w1 the first-order coefficients whose second moment
        // is exactly 1 in the stored precision, so the equilibrium carries exactly the momentum ρu
        // (rounded weights would give K ρu with K - 1 ~ 1e-8 in FP32, a drift growing with time).
        if constexpr (DEV) {
          feq[i] = p.w[i] * drho + rho * (p.w1[i] * cu + p.w[i] * eq_poly_hi<L>(p.cs, cu, usq));
        } else {
          const CT P = eq_poly<L>(p.cs, cu, usq);
          feq[i] = (rho * p.w[i]) * ((CT)1 + P);
        }
      }
      if constexpr (COLL == LBM_SRT) {
#pragma unroll
        for (int i = 0; i < L::Q; ++i) v[i] = p.om_a * v[i] + p.om_b * feq[i];
      } else {  // TRT
        CT out[L::Q];
#pragma unroll
        for (int i = 0; i < L::Q; ++i) {
          const int o = L::opp(i);
          const CT feq_s = (CT)0.5 * (feq[i] + feq[o]);
          const CT feq_a = (CT)0.5 * (feq[i] - feq[o]);
          const CT f_s = (CT)0.5 * (v[i] + v[o]);
          const CT f_a = (CT)0.5 * (v[i] - v[o]);
          out[i] = v[i] + (-p.inv_ts * (f_s - feq_s) - p.inv_ta * (f_a - feq_a));
        }
#pragma unroll
        for (int i = 0; i < L::Q; ++i) v[i] = out[i];
      }
    }
  }
}

// ---------------------------------------------------------------------------------------
// Kernels.  Grid: x blocks of 128 threads along x, one row of y per block row.
// ---------------------------------------------------------------------------------------
constexpr int kBlockX = 128;

// MODE 0: collide only (first step after an upload: f_stream -> f_collision)
// MODE 1: fused pull + boundaries + collide (post-collision -> post-collision)
// MODE 2: pull + boundaries only (post-collision -> f_stream, materialising the observable state)
template <class L, class S, int COLL, int MODE>
__global__ void __launch_bounds__(kBlockX) step_kernel(StepParams<typename S::C> p,
                                                       const typename S::T* __restrict__ src,
                                                       typename S::T* __restrict__ dst) {
  using CT = typename S::C;
  const int x = blockIdx.x * kBlockX + threadIdx.x;
  if (x >= p.nx) return;
  for (int y = blockIdx.y; y < p.ny; y += gridDim.y) {
    const int node = y * p.nx + x;
    if constexpr (COLL == LBM_MRT && MODE != 2) {
      // streaming form: populations feed the raw moments as they arrive, outputs are rebuilt
      // and stored one by one, so no per-node array of Q populations stays live
      CT M[15];
#pragma unroll
      for (int k = 0; k < 15; ++k) M[k] = 0;
      int xw[2 * L::R + 1], yo[2 * L::R + 1];
      bool near = false;
      if (MODE != 0) {
        pull_offsets<L>(p, x, y, xw, yo);
        near = p.nbc > 0 && (y < L::R || y >= p.ny - L::R || x < L::R || x >= p.nx - L::R);
      }
      auto pop = [&](int i) -> CT {
        if (MODE == 0) return S::ld(src + (size_t)i * p.n + node);
        return pop_streamed<L, S>(p, src, x, y, xw, yo, near, i);
      };
#pragma unroll
      for (int i = 0; i < L::Q; ++i) {
        const int o = L::opp(i);
        if (o == i) {
          M[0] += pop(i);
        } else if (o > i) {
          const CT a = pop(i), b = pop(o);
          mrt_accumulate_pair<L>(M, i, a + b, a - b);
        }
      }
      CT Fx = 0, Fy = 0;
      const bool has_force = p.force_kind != LBM_FORCE_NONE;
      if (has_force) node_force(p, x, y, Fx, Fy);
      MrtCoeffs<CT> c;
      mrt_coeffs<L, S::DEV>(p, M, Fx, Fy, has_force, c);
#pragma unroll
      for (int i = 0; i < L::Q; ++i) {
        const int o = L::opp(i);
        if (o == i) {
          S::st(dst + (size_t)i * p.n + node, p.w[i] * c.B[0]);
        } else if (o > i) {
          CT a, b;
          mrt_out_pair<L, S::DEV>(p, c, i, a, b);
          S::st(dst + (size_t)i * p.n + node, a);
          S::st(dst + (size_t)o * p.n + node, b);
        }
      }
    } else {
      CT v[L::Q];
      if (MODE == 0) load_local<L, S>(p, src, node, v);
      else load_streamed<L, S>(p, src, x, y, v);
      if (MODE != 2) collide_node<L, S, COLL>(p, x, y, v);
#pragma unroll
      for (int i = 0; i < L::Q; ++i) S::st(dst + (size_t)i * p.n + node, v[i]);
    }
  }
}

}  // namespace lbm
