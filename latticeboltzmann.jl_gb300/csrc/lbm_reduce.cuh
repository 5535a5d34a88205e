// lbm_reduce.cuh -- whole-lattice reductions for the processing methods (next!).
//
// Each kernel reads the populations of the state the reference's next!(pm, q, f_stream, t)
// observes: when the device holds the post-collision array, the periodic pull and the
// boundary conditions are applied on the fly (load_streamed), so no extra pass over the
// lattice is made.  Moments are formed in FP64 whatever the storage (deviation storage is
// widened as f = w + g), and the per-block partial sums are combined by a single block in
// a fixed order, so results are bitwise reproducible run to run.
#pragma once

#include "lbm_step.cuh"

namespace lbm {

constexpr int kRedThreads = 256;
// Blocks of a lattice-wide sum (reductions, the adjoint's parameter sums): a fixed partition, not
// one derived from the device's SM count, so that a sum's FP64 addition order, and so its bits,
// are the same on every device; 608 is four blocks per SM of a 152-SM GB300.
constexpr int kSumBlocks = 608;
constexpr int kRedMaxK = 16;

struct ReduceArgs {
  int kind;
  double w[LBM_MAX_Q];
  double cs;                        // 1 / c_s^2
  const double *rho_a, *ux_a, *uy_a, *p_a, *sxx_a, *syx_a, *sxy_a, *syy_a;  // analytic fields (device)
  double tau;                       // (1/c_s²)·ν for the stress estimate
  double u_max;
  double area;
  double* u_old;                    // VELOCITY_CONVERGENCE: 2 planes (device)
  int q_low_order;                  // D2Q4 / D2Q5: pressure(q, f, ρ, u) is the constant 1
};

template <int K>
__device__ __forceinline__ void block_reduce_store(double (&acc)[K], double* partial) {
  __shared__ double sh[kRedThreads / 32][K];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    double v = acc[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) sh[warp][k] = v;
  }
  __syncthreads();
  if (threadIdx.x < K) {
    double s = 0.0;
    for (int wi = 0; wi < kRedThreads / 32; ++wi) s += sh[wi][threadIdx.x];
    partial[(size_t)blockIdx.x * K + threadIdx.x] = s;
  }
}

// Per-node moments in FP64 of the observed populations.
template <class L, class S, bool PULL>
__device__ __forceinline__ void node_f64(const StepParams<typename S::C>& p, const ReduceArgs& r,
                                         const typename S::T* __restrict__ src, int x, int y, double* f) {
  using CT = typename S::C;
  CT v[L::Q];
  if (PULL) load_streamed<L, S>(p, src, x, y, v);
  else load_local<L, S>(p, src, y * p.nx + x, v);
#pragma unroll
  for (int i = 0; i < L::Q; ++i) f[i] = S::DEV ? r.w[i] + (double)v[i] : (double)v[i];
}

// An FP64 value whose +, - and * are the correctly rounded operations (__dadd_rn, __dsub_rn,
// __dmul_rn), which the compiler never fuses into FMAs: with plain expressions, whether a product
// is fused into the sum that consumes it depends on the code around it, so the same reduction could
// round differently in the single-lattice and the batched kernels that both inline it.  (The oracle,
// compiled without contraction, rounds every operation too.)
struct rd {
  double v;
  __device__ __forceinline__ rd(double x = 0.0) : v(x) {}
};
__device__ __forceinline__ rd operator+(rd a, rd b) { return rd(__dadd_rn(a.v, b.v)); }
__device__ __forceinline__ rd operator-(rd a, rd b) { return rd(__dsub_rn(a.v, b.v)); }
__device__ __forceinline__ rd operator*(rd a, rd b) { return rd(__dmul_rn(a.v, b.v)); }
__device__ __forceinline__ rd operator/(rd a, rd b) { return rd(a.v / b.v); }
__device__ __forceinline__ rd& operator+=(rd& a, rd b) { return a = a + b; }

// The contribution of node (x, y) to the K sums of one reduction kind.
template <class L, class S, bool PULL, int K>
__device__ __forceinline__ void reduce_node(const StepParams<typename S::C>& p, const ReduceArgs& r,
                                            const typename S::T* __restrict__ src, int x, int y, long long node,
                                            double (&acc)[K]) {
  auto add = [&](int k, rd t) { acc[k] = __dadd_rn(acc[k], t.v); };
  {
    const rd ics = 1.0 / r.cs;
    double fd[L::Q];
    node_f64<L, S, PULL>(p, r, src, x, y, fd);
    rd f[L::Q];
#pragma unroll
    for (int i = 0; i < L::Q; ++i) f[i] = fd[i];
    rd rho = f[0];
#pragma unroll
    for (int i = 1; i < L::Q; ++i) rho += f[i];
    rd jx = 0.0, jy = 0.0;
#pragma unroll
    for (int i = 0; i < L::Q; ++i) {
      jx += f[i] * (double)L::cx(i);
      jy += f[i] * (double)L::cy(i);
    }
    const rd ux = jx / rho, uy = jy / rho;
    if (K == 16) {  // TRACK_ERRORS, track_hydrodynamic_errors.jl:114-203
      rd axx = 0.0, axy = 0.0, ayy = 0.0;  // a_bar_2 = Σ f H_2(c)
#pragma unroll
      for (int i = 0; i < L::Q; ++i) {
        axx += f[i] * (rd((double)(L::cx(i) * L::cx(i))) - ics);
        axy += f[i] * (double)(L::cx(i) * L::cy(i));
        ayy += f[i] * (rd((double)(L::cy(i) * L::cy(i))) - ics);
      }
      const rd exx = rho * (ux * ux), exy = rho * (ux * uy), eyy = rho * (uy * uy);  // a_eq_2, T = 1
      const double tau = r.tau;
      const rd h = 1.0 / (2.0 * tau), den = 1.0 + 1.0 / (2.0 * tau);
      const rd A2xx = (axx + h * exx) / den, A2yy = (ayy + h * eyy) / den;
      const rd Pxx = A2xx - rho * (ux * ux - 1.0), Pyy = A2yy - rho * (uy * uy - 1.0);
      const rd pr = (Pxx + Pyy) / 2.0;
      // deviatoric_tensor(q, τ, f, ρ, u), moments.jl:81-96
      const rd sxx0 = (axx - exx) / den, sxy0 = (axy - exy) / den, syy0 = (ayy - eyy) / den;
      const rd tr = (sxx0 + syy0) / 2.0;
      const rd fac = 1.0 / (r.u_max * r.u_max);
      const rd sxx = (sxx0 - tr) * fac, sxy = sxy0 * fac, syy = (syy0 - tr) * fac, syx = sxy;
      const rd udx = ux / r.u_max, udy = uy / r.u_max;
      const size_t k = (size_t)node;
      const rd erho = r.rho_a[k], eux = r.ux_a[k], euy = r.uy_a[k], ep = r.p_a[k];
      const rd esxx = r.sxx_a[k], esyx = r.syx_a[k], esxy = r.sxy_a[k], esyy = r.syy_a[k];
      add(0, (rho - erho) * (rho - erho));
      add(1, (udx - eux) * (udx - eux) + (udy - euy) * (udy - euy));
      add(2, (pr - ep) * (pr - ep));
      add(3, (esxx - sxx) * (esxx - sxx));
      add(4, (esxy - sxy) * (esxy - sxy));
      add(5, (esyy - syy) * (esyy - syy));
      add(6, (esyx - syx) * (esyx - syx));
      add(7, eux * eux + euy * euy);
      add(8, esxx * esxx);
      add(9, esyy * esyy);
      add(10, esxy * esxy);
      add(11, esyx * esyx);
      add(12, ep * ep);
      add(13, rho);
      add(14, rho * (udx + udy));
      add(15, rho * (udx * udx + udy * udy));
    } else if (K == 12) {  // COMPARE, processing_methods.jl:177-239
      rd pr;
      if (r.q_low_order) {
        pr = 1.0;
      } else {
        rd axx = 0.0, ayy = 0.0;
#pragma unroll
        for (int i = 0; i < L::Q; ++i) {
          axx += f[i] * (rd((double)(L::cx(i) * L::cx(i))) - ics);
          ayy += f[i] * (rd((double)(L::cy(i) * L::cy(i))) - ics);
        }
        pr = ((axx + ayy) - rho * ((ux * ux + uy * uy) - 2.0)) / 2.0;  // moments.jl:21-33
      }
      const rd T = pr / rho;
      const rd udx = ux / r.u_max, udy = uy / r.u_max;
      const rd ke = (udx * udx + udy * udy) * rho;
      const size_t k = (size_t)node;
      const rd erho = r.rho_a[k], ep = r.p_a[k], eux = r.ux_a[k], euy = r.uy_a[k];
      const rd eT = ep / erho, eke = eux * eux + euy * euy;
      add(0, rho);
      add(1, (udx + udy) * rho);
      add(2, ke + T);
      add(3, ke);
      add(4, T);
      add(5, erho);
      add(6, erho * (eux + euy));
      add(7, eke + eT);
      add(8, eke);
      add(9, eT);
      add(10, rd(r.area) * ((udx - eux) * (udx - eux) + (udy - euy) * (udy - euy)));
      add(11, rd(r.area) * ((pr - ep) * (pr - ep)));
    } else if (K == 2) {  // MEAN_VELOCITY (stopping_criteria.jl:43-54)
      add(0, ux);
      add(1, 1.0);
    } else if (K == 3) {  // VELOCITY_CONVERGENCE (stopping_criteria.jl:101-116)
      const size_t k = (size_t)node;
      const rd ox = r.u_old[k], oy = r.u_old[p.n + k];
      add(0, (ux - ox) * (ux - ox) + (uy - oy) * (uy - oy));
      add(1, ox * ox + oy * oy);
      r.u_old[k] = ux.v;
      r.u_old[p.n + k] = uy.v;
    } else if (K == 4) {  // CONSERVED
      add(0, rho);
      add(1, jx);
      add(2, jy);
      int bad = 0;
#pragma unroll
      for (int i = 0; i < L::Q; ++i) bad += isfinite(fd[i]) ? 0 : 1;
      add(3, (double)bad);
    }
  }
}

template <class L, class S, bool PULL, int K>
__global__ void __launch_bounds__(kRedThreads) reduce_kernel(StepParams<typename S::C> p, ReduceArgs r,
                                                             const typename S::T* __restrict__ src,
                                                             double* __restrict__ partial) {
  double acc[K];
#pragma unroll
  for (int k = 0; k < K; ++k) acc[k] = 0.0;
  const long long first = (long long)blockIdx.x * kRedThreads + threadIdx.x, stride = (long long)gridDim.x * kRedThreads;
  NodeWalk w(first, stride, p.nx);
  for (long long node = first; node < p.n; node += stride, w.advance())
    reduce_node<L, S, PULL, K>(p, r, src, w.x, w.y, node, acc);
  block_reduce_store<K>(acc, partial);
}

// Sums the per-block partials in block order (deterministic).
template <int K>
__global__ void reduce_finish_kernel(const double* __restrict__ partial, int nblocks, double* __restrict__ out) {
  if (threadIdx.x < K) {
    double s = 0.0;
    for (int b = 0; b < nblocks; ++b) s += partial[(size_t)b * K + threadIdx.x];
    out[threadIdx.x] = s;
  }
}

// ρ, ux, uy planes of the observed state (density / velocity!, moments.jl:1-19).
template <class L, class S, bool PULL>
__global__ void __launch_bounds__(kBlockX) macro_kernel(StepParams<typename S::C> p, ReduceArgs r,
                                                        const typename S::T* __restrict__ src,
                                                        double* __restrict__ out) {
  const int x = blockIdx.x * kBlockX + threadIdx.x;
  if (x >= p.nx) return;
  for (int y = blockIdx.y; y < p.ny; y += gridDim.y) {
    double f[L::Q];
    node_f64<L, S, PULL>(p, r, src, x, y, f);
    double rho = f[0];
#pragma unroll
    for (int i = 1; i < L::Q; ++i) rho += f[i];
    double jx = 0.0, jy = 0.0;
#pragma unroll
    for (int i = 0; i < L::Q; ++i) {
      jx += f[i] * L::cx(i);
      jy += f[i] * L::cy(i);
    }
    const size_t k = (size_t)y * p.nx + x;
    out[k] = rho;
    out[p.n + k] = jx / rho;
    out[2 * p.n + k] = jy / rho;
  }
}

// Observed populations as FP64 planes (download of deviation storage, or materialisation).
template <class L, class S, bool PULL>
__global__ void __launch_bounds__(kBlockX) widen_kernel(StepParams<typename S::C> p, ReduceArgs r,
                                                        const typename S::T* __restrict__ src,
                                                        double* __restrict__ out) {
  const int x = blockIdx.x * kBlockX + threadIdx.x;
  if (x >= p.nx) return;
  for (int y = blockIdx.y; y < p.ny; y += gridDim.y) {
    double f[L::Q];
    node_f64<L, S, PULL>(p, r, src, x, y, f);
    const size_t k = (size_t)y * p.nx + x;
#pragma unroll
    for (int i = 0; i < L::Q; ++i) out[(size_t)i * p.n + k] = f[i];
  }
}

// FP64 planes -> storage (upload): f for F64, g = f - w (rounded once) for deviation storage.
template <class L, class S>
__global__ void __launch_bounds__(kBlockX) narrow_kernel(StepParams<typename S::C> p, ReduceArgs r,
                                                         const double* __restrict__ in,
                                                         typename S::T* __restrict__ dst) {
  const int x = blockIdx.x * kBlockX + threadIdx.x;
  if (x >= p.nx) return;
  for (int y = blockIdx.y; y < p.ny; y += gridDim.y) {
    const size_t k = (size_t)y * p.nx + x;
#pragma unroll
    for (int i = 0; i < L::Q; ++i) {
      const double f = in[(size_t)i * p.n + k];
      if constexpr (S::WIDE) dst[(size_t)i * p.n + k] = f;  // f itself, exactly
      else S::st(dst + (size_t)i * p.n + k, (typename S::C)(S::DEV ? f - r.w[i] : f));
    }
  }
}

// Macroscopic planes of the initial conditions (n doubles each, Julia layout; NULL = default).
struct InitFields {
  const double *rho, *ux, *uy, *T;  // defaults 1, 0, 0, 1
  const double *sxx, *sxy, *syy;    // symmetric stress-term tensor S (all NULL: no stress term)
  double coef;                      // stress-term coefficient
  int times_rho;                    // the stress term is also multiplied by ρ
};

// Initial populations from macroscopic fields, in FP64 whatever the storage
// (src/initial_conditions/*.jl):
//   f_i = w_i (ρ + Σ_{n=1..N} a_eq^(n)(ρ, u, T) : H_n(c_i) / (n! c_s^{2n}))
// the Hermite equilibrium `equilibrium(q, ρ, u, T)` of hermite.jl:10-33 (N = order(q) ÷ 2,
// a_eq^(n) of hermite.jl:37-77 including its repeated δ(b,d) / δ(a,d) terms at n = 4, H_n of
// hermite_polynomials.jl:47-82 with c_s² in the isotropic terms; tensor sums in column-major
// order), plus the stress term coef [ρ] w_i H_2(c_i) : S of analytical_offequilibrium.jl:10-87
// and analytical_velocity_stress.jl.
template <class L, class S>
__global__ void __launch_bounds__(kBlockX) init_fields_kernel(StepParams<typename S::C> p, ReduceArgs r,
                                                              InitFields in, typename S::T* __restrict__ dst) {
  const int x = blockIdx.x * kBlockX + threadIdx.x;
  if (x >= p.nx) return;
  const double css = 1.0 / r.cs;  // c_s²
  for (int y = blockIdx.y; y < p.ny; y += gridDim.y) {
    const size_t k = (size_t)y * p.nx + x;
    const double rho = in.rho ? in.rho[k] : 1.0;
    const double u[2] = {in.ux ? in.ux[k] : 0.0, in.uy ? in.uy[k] : 0.0};
    const double T = in.T ? in.T[k] : 1.0;
    const double lam = css * (T - 1.0), lam2 = (css * css) * ((T - 1.0) * (T - 1.0));
    auto d = [](int a, int b) { return a == b ? 1.0 : 0.0; };
    double a1[2], a2[2][2], a3[2][2][2], a4[2][2][2][2];
#pragma unroll
    for (int a = 0; a < 2; ++a) a1[a] = rho * u[a];
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
      for (int b = 0; b < 2; ++b) a2[a][b] = rho * (a == b ? u[a] * u[b] + lam : u[a] * u[b]);
    if constexpr (L::HN >= 3) {
#pragma unroll
      for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 2; ++b)
#pragma unroll
          for (int c = 0; c < 2; ++c)
            a3[a][b][c] = rho * (u[a] * u[b] * u[c] + lam * ((u[a] * d(b, c) + u[b] * d(a, c)) + u[c] * d(a, b)));
    }
    if constexpr (L::HN >= 4) {
#pragma unroll
      for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 2; ++b)
#pragma unroll
          for (int c = 0; c < 2; ++c)
#pragma unroll
            for (int e = 0; e < 2; ++e)
              a4[a][b][c][e] = rho * (u[a] * u[b] * u[c] * u[e] +
                                      lam * (u[a] * u[b] * d(c, e) + u[a] * u[c] * d(b, e) + u[a] * u[e] * d(b, e) +
                                             u[b] * u[c] * d(a, e) + u[b] * u[e] * d(a, e) + u[c] * u[e] * d(a, b)) +
                                      lam2 * (d(a, b) * d(c, e) + d(a, c) * d(b, e) + d(a, e) * d(b, c)));
    }
    static_for<0, L::Q>([&](auto I) {
      constexpr int i = decltype(I)::value;
      const double cv[2] = {(double)L::cx(i), (double)L::cy(i)};
      double acc = 0.0 + a1[0] * cv[0];
      acc = acc + a1[1] * cv[1];
      double s = acc / css;
      if constexpr (L::HN >= 2) {
        acc = 0.0;
#pragma unroll
        for (int b = 0; b < 2; ++b)
#pragma unroll
          for (int a = 0; a < 2; ++a) acc = acc + a2[a][b] * (cv[b] * cv[a] - css * d(a, b));
        s = s + acc / (2.0 * (css * css));
      }
      if constexpr (L::HN >= 3) {
        acc = 0.0;
#pragma unroll
        for (int c = 0; c < 2; ++c)
#pragma unroll
          for (int b = 0; b < 2; ++b)
#pragma unroll
            for (int a = 0; a < 2; ++a)
              acc = acc + a3[a][b][c] * (cv[c] * cv[b] * cv[a] -
                                         css * (cv[a] * d(b, c) + cv[b] * d(a, c) + cv[c] * d(a, b)));
        s = s + acc / (6.0 * (css * css * css));
      }
      if constexpr (L::HN >= 4) {
        acc = 0.0;
#pragma unroll
        for (int e = 0; e < 2; ++e)
#pragma unroll
          for (int c = 0; c < 2; ++c)
#pragma unroll
            for (int b = 0; b < 2; ++b)
#pragma unroll
              for (int a = 0; a < 2; ++a) {
                const double H = cv[e] * cv[c] * cv[b] * cv[a] -
                                 css * (cv[a] * cv[b] * d(c, e) + cv[a] * cv[c] * d(b, e) + cv[a] * cv[e] * d(b, c) +
                                        cv[b] * cv[c] * d(a, e) + cv[b] * cv[e] * d(a, c) + cv[c] * cv[e] * d(a, b)) +
                                 (css * css) * (d(a, b) * d(c, e) + d(a, c) * d(b, e) + d(a, e) * d(b, c));
                acc = acc + a4[a][b][c][e] * H;
              }
        s = s + acc / (24.0 * (css * css * css * css));
      }
      double f = r.w[i] * (rho + s);
      if (in.sxx) {
        const double HS = (cv[0] * cv[0] - css) * in.sxx[k] + (cv[1] * cv[0]) * in.sxy[k] +
                          (cv[0] * cv[1]) * in.sxy[k] + (cv[1] * cv[1] - css) * in.syy[k];
        f = f + (in.coef * (in.times_rho ? rho : 1.0)) * r.w[i] * HS;
      }
      if constexpr (S::WIDE) dst[(size_t)i * p.n + k] = f;  // f itself, exactly
      else S::st(dst + (size_t)i * p.n + k, (typename S::C)(S::DEV ? f - r.w[i] : f));
    });
  }
}

// Density of one node of the observed state (DensityConvergence, density_convergence.jl:6-17).
template <class L, class S, bool PULL>
__global__ void node_density_kernel(StepParams<typename S::C> p, ReduceArgs r, const typename S::T* __restrict__ src,
                                    int x, int y, double* __restrict__ out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double f[L::Q];
  node_f64<L, S, PULL>(p, r, src, x, y, f);
  double rho = f[0];
#pragma unroll
  for (int i = 1; i < L::Q; ++i) rho += f[i];
  out[0] = rho;
}

// apply!(bcs, q, f_new, f_old) on FP64 arrays in place (the single-operator entry point).
template <class L>
__global__ void __launch_bounds__(kBlockX) apply_bcs_kernel(StepParams<double> p, double* __restrict__ fnew,
                                                            const double* __restrict__ fold) {
  const int x = blockIdx.x * kBlockX + threadIdx.x;
  if (x >= p.nx) return;
  for (int y = blockIdx.y; y < p.ny; y += gridDim.y) {
  if (!(y < L::R || y >= p.ny - L::R || x < L::R || x >= p.nx - L::R)) continue;
  const int node = y * p.nx + x;
  const int y1 = y + 1, x1 = x + 1;
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
        if (hit) fnew[(size_t)i * p.n + node] = fold[(size_t)o * p.n + node];
      }
    } else {
#pragma unroll
      for (int i = 0; i < L::Q; ++i) {
        const int o = L::opp(i);
        if (y1 + L::cy(o) > p.ny) fnew[(size_t)i * p.n + node] = fold[(size_t)o * p.n + node] + bc.add[i];
      }
    }
  }
  }
}

}  // namespace lbm
