// lbm_adjoint.cuh -- reverse-mode (adjoint) kernels of the fused collide-stream step.
//
// The reference has no differentiation; this is the discrete adjoint of the forward map the
// kernels implement, for lattices with SRT, TRT or (second-order sets) regularised MRT collision, a
// uniform force and the boundary conditions (bounce-back, moving wall):
//
//   A_{t+1} = S C(A_t; τ_s, τ_a, F),  A_0 = f_eq(ρ = 1, u0),  L = Σ_x |u(A_T) - u*|²,
//
// with S the periodic pull followed by the boundary rules (each population taken from one source:
// a neighbour, or the same node's opposite population where a wall replaces it; a moving wall adds
// a constant) and C the per-node collision.  The adjoint state λ_t = ∂L/∂A_t obeys
// λ_t = J_C(A_t)^T S^T λ_{t+1}: S^T sends each λ back to its population's source (λ from x + c_i,
// and at a wall the swap of opposite populations), and J_C^T is applied per node in O(Q):
//
//   C(f) = M f + N f_eq(ρ(f), u'(f)),   M = (1-ω_s) P_s + (1-ω_a) P_a,   N = ω_s P_s + ω_a P_a,
//   J_C^T μ = M μ + (∂f_eq/∂f)^T ν,  ν = N μ,
//   (∂f_eq/∂f)^T ν |_k = G_ρ + Σ_a G_a (c_ka - u_a) / ρ,
//   G_ρ = Σ_i ν_i f_eq,i / ρ,   G_a = Σ_i ν_i ∂f_eq,i/∂u'_a,   u' = u + τ_a F,
//
// where P_s / P_a are the symmetric / antisymmetric parts over opposite pairs (trt.jl:71-94).
// Parameter sensitivities accumulate μ^T ∂C/∂θ per node: -Σ μ^s (f - f_eq) for ω_s,
// -Σ μ^a (f - f_eq) for ω_a, Σ_a G_a F_a for τ_a through the force shift, τ_a G_a for F_a.
// The MRT collision's transpose is formed through its moments instead (adj_mrt_node).
// Sums are FP64, one slot per block, blocks always own the same nodes (deterministic).
#pragma once

#include "lbm_step.cuh"

namespace lbm {

constexpr int kAdjThreads = 256;
constexpr int kAdjParams = 5;  // dω_s, dω_a, dτ_a (force shift), dF_x, dF_y

struct AdjArgs {
  double Fx, Fy;        // uniform lattice force
  double shift;         // τ (SRT) or τ_a (TRT)
};

// Equilibrium of one node as the forward kernel forms it, with ∂feq_i/∂u'_a.
// F64: feq = ρ w (1 + P);  deviation: geq = feq - w = w δρ + ρ (w1 c·u' + w P_2).
template <class L, class S>
__device__ __forceinline__ void adj_equilibrium(const StepParams<typename S::C>& p, typename S::C rho,
                                                typename S::C drho, typename S::C ux, typename S::C uy,
                                                typename S::C* feq, typename S::C* dfx, typename S::C* dfy) {
  using CT = typename S::C;
  const CT cs = p.cs;
  const CT usq = ux * ux + uy * uy;
  static_for<0, L::Q>([&](auto I) {
    constexpr int i = decltype(I)::value;
    constexpr CT cxi = (CT)L::cx(i), cyi = (CT)L::cy(i);
    const CT cu = cxi * ux + cyi * uy;
    const CT P2 = (CT)0.5 * (cs * cs * cu * cu - cs * usq);
    if constexpr (S::DEV) {
      feq[i] = p.w[i] * drho + rho * (p.w1[i] * cu + p.w[i] * P2);
      dfx[i] = rho * (p.w1[i] * cxi + p.w[i] * (cs * cs * cu * cxi - cs * ux));
      dfy[i] = rho * (p.w1[i] * cyi + p.w[i] * (cs * cs * cu * cyi - cs * uy));
    } else {
      feq[i] = (rho * p.w[i]) * ((CT)1 + cs * cu + P2);
      dfx[i] = rho * p.w[i] * (cs * cxi + cs * cs * cu * cxi - cs * ux);
      dfy[i] = rho * p.w[i] * (cs * cyi + cs * cs * cu * cyi - cs * uy);
    }
  });
}

// Adds the block's sums of K values to its slots: every thread's values go to shared memory and
// one warp adds them in a fixed order (a per-thread shuffle tree would cost 5 FP64 additions per
// value and thread on a GPU that issues two FP64 instructions per SM per clock).
template <int K>
__device__ __forceinline__ void adj_block_add(double (&acc)[K], double* slots) {
  __shared__ double sh[K][kAdjThreads];
#pragma unroll
  for (int k = 0; k < K; ++k) sh[k][threadIdx.x] = acc[k];
  __syncthreads();
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
#pragma unroll
    for (int k = 0; k < K; ++k) {
      double v = sh[k][lane];
      for (int j = lane + 32; j < kAdjThreads; j += 32) v += sh[k][j];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
      if (lane == 0) slots[(size_t)blockIdx.x * K + k] += v;
    }
  }
}

// A_0 = f_eq(ρ = 1, u0) in the storage's form.
template <class L, class S>
__global__ void __launch_bounds__(kAdjThreads) adj_init_kernel(StepParams<typename S::C> p, const double* __restrict__ u0,
                                                               typename S::T* __restrict__ a0) {
  using CT = typename S::C;
  for (long long node = (long long)blockIdx.x * kAdjThreads + threadIdx.x; node < p.n;
       node += (long long)gridDim.x * kAdjThreads) {
    const CT ux = (CT)u0[node], uy = (CT)u0[p.n + node];
    CT feq[L::Q], dfx[L::Q], dfy[L::Q];
    adj_equilibrium<L, S>(p, (CT)1, (CT)0, ux, uy, feq, dfx, dfy);
#pragma unroll
    for (int i = 0; i < L::Q; ++i) S::st(a0 + (size_t)i * p.n + node, feq[i]);
  }
}

// Loss L = Σ |u(A_T) - u*|² (FP64) and λ_T = ∂L/∂A_T, with A_T pulled from B_{T-1}.
template <class L, class S>
__global__ void __launch_bounds__(kAdjThreads) adj_loss_kernel(StepParams<typename S::C> p, const typename S::T* __restrict__ src,
                                                               const double* __restrict__ ut, typename S::T* __restrict__ lam,
                                                               double* __restrict__ slots) {
  using CT = typename S::C;
  double acc[1] = {0.0};
  const long long first = (long long)blockIdx.x * kAdjThreads + threadIdx.x, stride = (long long)gridDim.x * kAdjThreads;
  NodeWalk w(first, stride, p.nx);
  for (long long node = first; node < p.n; node += stride, w.advance()) {
    const int y = w.y, x = w.x;
    CT v[L::Q];
    load_streamed<L, S>(p, src, x, y, v);
    double rho = 0.0, jx = 0.0, jy = 0.0;
#pragma unroll
    for (int i = 0; i < L::Q; ++i) {
      const double f = S::DEV ? (double)p.w[i] + (double)v[i] : (double)v[i];
      rho += f;
      jx += f * L::cx(i);
      jy += f * L::cy(i);
    }
    const double ux = jx / rho, uy = jy / rho;
    const double ex = ux - ut[node], ey = uy - ut[p.n + node];
    acc[0] += ex * ex + ey * ey;
#pragma unroll
    for (int i = 0; i < L::Q; ++i) {
      const double g = 2.0 * (ex * (L::cx(i) - ux) + ey * (L::cy(i) - uy)) / rho;
      lam[(size_t)i * p.n + node] = (typename S::T)g;
    }
  }
  adj_block_add<1>(acc, slots);
}

// Whether the boundary conditions replace population i of node (x, y) in the pull (the rule of
// load_streamed: bounce_back.jl:8-72, moving_wall.jl:17-38).  A replaced population is the same
// node's post-collision opposite population (plus a constant for a moving wall), whichever of the
// listed conditions replaces it last.
template <class L, class CT>
__device__ __forceinline__ bool bc_replaces(const StepParams<CT>& p, int x, int y, int i) {
  const int o = L::opp(i);
  const int y1 = y + 1, x1 = x + 1;
  for (int b = 0; b < p.nbc; ++b) {
    const BCDev& bc = p.bc[b];
    if (bc.kind == LBM_BOUNCE_BACK) {
      if (x < bc.x_lo || x > bc.x_hi || y < bc.y_lo || y > bc.y_hi) continue;
      bool hit;
      if (bc.dir == LBM_NORTH) hit = y1 + L::cy(o) > p.ny;
      else if (bc.dir == LBM_SOUTH) hit = y1 + L::cy(o) <= 0;
      else if (bc.dir == LBM_EAST) hit = x1 + L::cx(o) > p.nx;
      else hit = x1 + L::cx(o) <= 0;
      if (hit) return true;
    } else if (y1 + L::cy(o) > p.ny) {
      return true;
    }
  }
  return false;
}

// J_C^T μ of the regularised MRT collision of a second-order set (mrt.jl:56-118 with N = 2), in
// the form the forward kernel evaluates it (mrt_coeffs):
//   M_ab = Σ_i f_i c_x^a c_y^b,  ρ = M_00 (+1 in deviation form),  u' = M_1/ρ + τ_2 F,
//   X = M_2 - M_00 I / κ (the Hermite coefficient a_f),  E = ρ u'u' (a_eq),  A = (1-ω) X + ω E,
//   f_out,i = w_i (M_00 - κ tr A / 2 + κ²/2 (A_xx c_x² + 2 A_xy c_x c_y + A_yy c_y²))
//             + W1_i (c_x ρu'_x + c_y ρu'_y),
// with ω = 1/τ_2, κ = 1/c_s² (the reference's speed_of_sound_squared), W1_i = κ w_i (FP64) or the
// momentum-exact w1_i (deviation form).  Reverse:
// Λ = Σ_i μ_i w_i (1, c_x², c_x c_y, c_y²) and Σ_i μ_i W1_i c_i give ∂L/∂A, ∂L/∂(ρu'), then
// ∂L/∂M_ab through ρ, u' and X, and λ_i = Σ_ab ∂L/∂M_ab c_x^a c_y^b.  Parameters: ∂A/∂ω = E - X
// (slot 0), ∂u'/∂τ_2 = F through the force shift (slot 2), ∂u'/∂F = τ_2 (slots 3, 4).
template <class L, class S>
__device__ __forceinline__ void adj_mrt_node(const StepParams<typename S::C>& p, const typename S::C* f,
                                             const typename S::C* mu, typename S::C Fx, typename S::C Fy,
                                             typename S::C shift, typename S::C sFx, typename S::C sFy,
                                             typename S::C* tacc, typename S::T* __restrict__ lam_out, long long node) {
  static_assert(L::HN == 2, "the MRT adjoint covers second-order velocity sets");
  using CT = typename S::C;
  CT M0 = 0, M1 = 0, M2 = 0, M3 = 0, M4 = 0, M5 = 0;
  CT L0 = 0, L3 = 0, L4 = 0, L5 = 0, Lx = 0, Ly = 0;
  static_for<0, L::Q>([&](auto I) {
    constexpr int i = decltype(I)::value;
    constexpr CT cx = (CT)L::cx(i), cy = (CT)L::cy(i);
    M0 += f[i];
    M1 += cx * f[i];
    M2 += cy * f[i];
    M3 += (cx * cx) * f[i];
    M4 += (cx * cy) * f[i];
    M5 += (cy * cy) * f[i];
    const CT wm = p.w[i] * mu[i];
    const CT w1m = (S::DEV ? p.w1[i] : p.w[i] * p.cs) * mu[i];
    L0 += wm;
    L3 += (cx * cx) * wm;
    L4 += (cx * cy) * wm;
    L5 += (cy * cy) * wm;
    Lx += cx * w1m;
    Ly += cy * w1m;
  });
  const CT rho = S::DEV ? (CT)1 + M0 : M0;
  const CT inv_rho = (CT)1 / rho;
  const CT vx = M1 * inv_rho, vy = M2 * inv_rho;
  const CT ux = vx + sFx, uy = vy + sFy;
  const CT om = p.mrt_b[1], am = p.mrt_a[1];
  const CT ics = (CT)1 / p.cs, c2 = p.cs * p.cs * (CT)0.5;
  const CT gxx = c2 * (L3 - ics * L0), gyy = c2 * (L5 - ics * L0), gxy = (CT)2 * c2 * L4;
  tacc[0] += gxx * (rho * ux * ux - (M3 - ics * M0)) + gxy * (rho * ux * uy - M4) + gyy * (rho * uy * uy - (M5 - ics * M0));
  const CT gux = om * rho * ((CT)2 * ux * gxx + uy * gxy) + rho * Lx;
  const CT guy = om * rho * (ux * gxy + (CT)2 * uy * gyy) + rho * Ly;
  const CT grho = om * (ux * ux * gxx + ux * uy * gxy + uy * uy * gyy) + ux * Lx + uy * Ly -
                  (gux * vx + guy * vy) * inv_rho;
  const CT gM0 = L0 - am * ics * (gxx + gyy) + grho;
  const CT gM1 = gux * inv_rho, gM2 = guy * inv_rho, gM3 = am * gxx, gM4 = am * gxy, gM5 = am * gyy;
  tacc[2] += gux * Fx + guy * Fy;
  tacc[3] += shift * gux;
  tacc[4] += shift * guy;
  static_for<0, L::Q>([&](auto I) {
    constexpr int i = decltype(I)::value;
    constexpr CT cx = (CT)L::cx(i), cy = (CT)L::cy(i);
    const CT l = gM0 + gM1 * cx + gM2 * cy + gM3 * (cx * cx) + gM4 * (cx * cy) + gM5 * (cy * cy);
    lam_out[(size_t)i * p.n + node] = (typename S::T)l;
  });
}

// One reverse step: λ_t = J_C(A_t)^T S^T λ_{t+1}.  A_t is pulled from B_{t-1} (pull = true) or
// read locally (A_0).  Parameter sensitivities are added to this block's slots.
template <class L, class S, int COLL>
__global__ void __launch_bounds__(kAdjThreads, (S::DEV && L::Q <= 9) ? 4 : 1) adj_step_kernel(StepParams<typename S::C> p, AdjArgs a,
                                                               const typename S::T* __restrict__ src, int pull,
                                                               const typename S::T* __restrict__ lam_next,
                                                               typename S::T* __restrict__ lam_out,
                                                               double* __restrict__ slots) {
  using CT = typename S::C;
  wait_prior_grid();  // launched after the previous step's kernel (launch_after_prior)
  // per-thread sums in the compute type (a thread owns about two nodes), widened to FP64 once
  // for the block's fixed-order FP64 sum: no FP64 instruction per node
  CT tacc[kAdjParams] = {0, 0, 0, 0, 0};
  const CT om_s = COLL == LBM_TRT ? p.inv_ts : p.om_b;
  const CT om_a = COLL == LBM_TRT ? p.inv_ta : p.om_b;
  const CT Fx = (CT)a.Fx, Fy = (CT)a.Fy, shift = (CT)a.shift;
  const CT sFx = (CT)(a.shift * a.Fx), sFy = (CT)(a.shift * a.Fy);
  const long long first = (long long)blockIdx.x * kAdjThreads + threadIdx.x, stride = (long long)gridDim.x * kAdjThreads;
  NodeWalk w(first, stride, p.nx);
  for (long long node = first; node < p.n; node += stride, w.advance()) {
    const int y = w.y, x = w.x;
    // forward state A_t at the node
    CT f[L::Q];
    if (pull) load_streamed<L, S>(p, src, x, y, f);
    else load_local<L, S>(p, src, (int)node, f);
    // μ = S^T λ_{t+1}: λ from x + c_i (the opposite of the forward pull).  With boundary
    // conditions, population i of x + c_i pulls from x only where no condition replaces it, and a
    // population replaced at x itself (the opposite of i, read from this node) sends its λ here;
    // both can only happen within 2R of an edge.
    CT mu[L::Q];
    {
      int xw[2 * L::R + 1], yo[2 * L::R + 1];
      pull_offsets<L>(p, x, y, xw, yo);
      const bool near = p.nbc > 0 && (y < 2 * L::R || y >= p.ny - 2 * L::R || x < 2 * L::R || x >= p.nx - 2 * L::R);
      static_for<0, L::Q>([&](auto I) {
        constexpr int i = decltype(I)::value;
        const size_t from = (size_t)i * p.n + yo[L::R - L::cy(i)] + xw[L::R - L::cx(i)];
        if (!near) {
          mu[i] = (CT)lam_next[from];
        } else {
          int xt = x - p.dxm[3 - L::cx(i)], yt = y - p.dym[3 - L::cy(i)];  // x + c_i, periodic
          xt += xt < 0 ? p.nx : 0;
          yt += yt < 0 ? p.ny : 0;
          CT m = 0;
          if (!bc_replaces<L>(p, xt, yt, i)) m = (CT)lam_next[from];
          constexpr int o = L::opp(i);
          if (bc_replaces<L>(p, x, y, o)) m = m + (CT)lam_next[(size_t)o * p.n + (size_t)y * p.nx + x];
          mu[i] = m;
        }
      });
    }
    if constexpr (COLL == LBM_MRT) {
      adj_mrt_node<L, S>(p, f, mu, Fx, Fy, shift, sFx, sFy, tacc, lam_out, node);
      continue;
    }
    // moments, equilibrium and its velocity derivatives (as the forward collision forms them)
    CT s = 0, jx = 0, jy = 0;
    static_for<0, L::Q>([&](auto I) {
      constexpr int i = decltype(I)::value;
      s += f[i];
      jx += (CT)L::cx(i) * f[i];
      jy += (CT)L::cy(i) * f[i];
    });
    const CT rho = S::DEV ? (CT)1 + s : s;
    const CT drho = s;
    const CT inv_rho = (CT)1 / rho;
    const CT ux = jx * inv_rho, uy = jy * inv_rho;
    const CT upx = ux + sFx, upy = uy + sFy;
    CT feq[L::Q], dfx[L::Q], dfy[L::Q];
    adj_equilibrium<L, S>(p, rho, drho, upx, upy, feq, dfx, dfy);
    // ν = N μ and M μ per opposite pair
    CT nu[L::Q], Mmu[L::Q];
    static_for<0, L::Q>([&](auto I) {
      constexpr int i = decltype(I)::value, o = L::opp(i);
      const CT ms = (CT)0.5 * (mu[i] + mu[o]), ma = (CT)0.5 * (mu[i] - mu[o]);
      nu[i] = om_s * ms + om_a * ma;
      Mmu[i] = ((CT)1 - om_s) * ms + ((CT)1 - om_a) * ma;
      const CT fneq = f[i] - feq[i];  // deviation storage: g - geq
      tacc[0] -= ms * fneq;
      tacc[1] -= ma * fneq;
    });
    CT Grho = 0, Gx = 0, Gy = 0;
    static_for<0, L::Q>([&](auto I) {
      constexpr int i = decltype(I)::value;
      const CT fe = S::DEV ? feq[i] + p.w[i] : feq[i];
      Grho += nu[i] * fe;
      Gx += nu[i] * dfx[i];
      Gy += nu[i] * dfy[i];
    });
    Grho = Grho * inv_rho;
    tacc[2] += Gx * Fx + Gy * Fy;
    tacc[3] += shift * Gx;
    tacc[4] += shift * Gy;
    const CT gx = Gx * inv_rho, gy = Gy * inv_rho, base = Grho - (gx * ux + gy * uy);
    static_for<0, L::Q>([&](auto I) {
      constexpr int i = decltype(I)::value;
      constexpr CT cxi = (CT)L::cx(i), cyi = (CT)L::cy(i);
      const CT l = Mmu[i] + base + (gx * cxi + gy * cyi);
      lam_out[(size_t)i * p.n + node] = (typename S::T)l;
    });
  }
  double acc[kAdjParams];
#pragma unroll
  for (int k = 0; k < kAdjParams; ++k) acc[k] = (double)tacc[k];
  adj_block_add<kAdjParams>(acc, slots);
}

// ∂L/∂u0 = (∂A_0/∂u0)^T λ_0 per node, FP64 output planes.
template <class L, class S>
__global__ void __launch_bounds__(kAdjThreads) adj_u0_kernel(StepParams<typename S::C> p, const double* __restrict__ u0,
                                                             const typename S::T* __restrict__ lam0,
                                                             double* __restrict__ grad) {
  using CT = typename S::C;
  for (long long node = (long long)blockIdx.x * kAdjThreads + threadIdx.x; node < p.n;
       node += (long long)gridDim.x * kAdjThreads) {
    const CT ux = (CT)u0[node], uy = (CT)u0[p.n + node];
    CT feq[L::Q], dfx[L::Q], dfy[L::Q];
    adj_equilibrium<L, S>(p, (CT)1, (CT)0, ux, uy, feq, dfx, dfy);
    double gx = 0.0, gy = 0.0;
#pragma unroll
    for (int i = 0; i < L::Q; ++i) {
      const double l = (double)(CT)lam0[(size_t)i * p.n + node];
      gx += l * (double)dfx[i];
      gy += l * (double)dfy[i];
    }
    grad[node] = gx;
    grad[p.n + node] = gy;
  }
}

template <int K>
__global__ void adj_finish_kernel(const double* __restrict__ slots, int nblocks, double* __restrict__ out) {
  if (threadIdx.x < K) {
    double s = 0.0;
    for (int b = 0; b < nblocks; ++b) s += slots[(size_t)b * K + threadIdx.x];
    out[threadIdx.x] = s;
  }
}

}  // namespace lbm
