// lbm_oracle.cpp -- CPU restatement of LatticeBoltzmann.jl's collide-stream hot path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the oracle for the CUDA path: only the
// test-suite, the smoke check and the CPU-baseline leg of the benchmark load it.  The
// product (liblbm_gb300.so) never links, calls or falls back to it.
//
// Every function follows the reference algorithm step by step, in the reference's own
// loop order and with the same arithmetic expression structure, so that rounding stays
// close to the Julia code (compiled with -ffp-contract=off: no fused multiply-adds, as in
// Julia without @fastmath).  Citations are file:line inside the reference project.
//
// Layout: every lattice array is the Julia array f[x, y, i] in column-major order, i.e.
// f[x + nx * (y + ny * i)] with 0-based x, y, i.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc {

// ---------------------------------------------------------------------------------------
// L0: quadratures (src/quadratures.jl, src/quadratures/D2Q*.jl)
// ---------------------------------------------------------------------------------------
enum QuadId { Q_D2Q4 = 0, Q_D2Q5, Q_D2Q9, Q_D2Q13, Q_D2Q17, Q_D2Q21, Q_D2Q37 };

struct Quad {
  int id = 0, Q = 0, order = 0;
  int cx[37] = {0}, cy[37] = {0};
  double w[37] = {0};
  double cs = 0;  // the reference field `speed_of_sound_squared`, which holds 1 / c_s^2
};

static void set_c(Quad& q, std::initializer_list<int> xs, std::initializer_list<int> ys) {
  int i = 0;
  for (int v : xs) q.cx[i++] = v;
  q.Q = i;
  i = 0;
  for (int v : ys) q.cy[i++] = v;
}

static Quad make_quad(int id) {
  Quad q;
  q.id = id;
  switch (id) {
    case Q_D2Q4:  // src/quadratures/D2Q4.jl:16-24
      set_c(q, {1, 0, -1, 0}, {0, 1, 0, -1});
      for (int i = 0; i < 4; ++i) q.w[i] = 1.0 / 4.0;
      q.cs = 2.0;
      q.order = 3;
      break;
    case Q_D2Q5:  // src/quadratures/D2Q5.jl:17-31
      set_c(q, {0, 1, 0, -1, 0}, {0, 0, 1, 0, -1});
      q.w[0] = 4.0 / 6.0;
      for (int i = 1; i < 5; ++i) q.w[i] = 1.0 / 12.0;
      q.cs = 6.0;
      q.order = 3;
      break;
    case Q_D2Q9: {  // src/quadratures/D2Q9.jl:20-27
      set_c(q, {0, -1, -1, -1, 0, 1, 1, 1, 0}, {0, 1, 0, -1, -1, -1, 0, 1, 1});
      const double w[9] = {4.0 / 9.0, 1.0 / 36.0, 1.0 / 9.0, 1.0 / 36.0, 1.0 / 9.0,
                           1.0 / 36.0, 1.0 / 9.0, 1.0 / 36.0, 1.0 / 9.0};
      for (int i = 0; i < 9; ++i) q.w[i] = w[i];
      q.cs = 3.0;
      q.order = 5;
      break;
    }
    case Q_D2Q13: {  // src/quadratures/D2Q13.jl:10-27
      set_c(q, {0, 1, -1, 0, 0, 1, -1, 1, -1, 2, -2, 0, 0},
            {0, 0, 0, 1, -1, 1, -1, -1, 1, 0, 0, -2, 2});
      const double w0 = 3.0 / 8.0, w1 = 1.0 / 12.0, w2 = 1.0 / 16.0, w3 = 1.0 / 96.0;
      const double w[13] = {w0, w1, w1, w1, w1, w2, w2, w2, w2, w3, w3, w3, w3};
      for (int i = 0; i < 13; ++i) q.w[i] = w[i];
      q.cs = 2.0;
      q.order = 5;
      break;
    }
    case Q_D2Q17: {  // src/quadratures/D2Q17.jl:21-57
      set_c(q, {0, 1, -1, 0, 0, 1, -1, 1, -1, 2, -2, 2, -2, 3, -3, 0, 0},
            {0, 0, 0, 1, -1, 1, -1, -1, 1, 2, -2, -2, 2, 0, 0, 3, -3});
      const double sq = std::sqrt(193.0);
      const double w0 = (575.0 + 193.0 * sq) / 8100.0;
      const double w1 = (3355.0 - 91.0 * sq) / 18000.0;
      const double w2 = (655.0 + 17.0 * sq) / 27000.0;
      const double w3 = (685.0 - 49.0 * sq) / 54000.0;
      const double w4 = (1445.0 - 101.0 * sq) / 162000.0;
      const double w[17] = {w0, w1, w1, w1, w1, w2, w2, w2, w2, w3, w3, w3, w3, w4, w4, w4, w4};
      for (int i = 0; i < 17; ++i) q.w[i] = w[i];
      q.cs = (125.0 + 5.0 * std::sqrt(193.0)) / 72.0;
      q.order = 7;
      break;
    }
    case Q_D2Q21: {  // src/quadratures/D2Q21.jl:15-71 (25 velocities; the last four weigh 0)
      set_c(q, {0, 1, -1, 0, 0, 1, -1, 1, -1, 2, -2, 0, 0, 2, -2, 2, -2, 3, -3, 0, 0, 3, -3, -3, 3},
            {0, 0, 0, 1, -1, 1, -1, -1, 1, 0, 0, 2, -2, 2, -2, -2, 2, 0, 0, 3, -3, 3, -3, 3, -3});
      const double w0 = 91.0 / 324.0, w1 = 1.0 / 12.0, w2 = 2.0 / 27.0, w3 = 7.0 / 360.0,
                   w4 = 1.0 / 432.0, w5 = 1.0 / 1620.0, w6 = 0.0;
      const double w[25] = {w0, w1, w1, w1, w1, w2, w2, w2, w2, w3, w3, w3, w3,
                            w4, w4, w4, w4, w5, w5, w5, w5, w6, w6, w6, w6};
      for (int i = 0; i < 25; ++i) q.w[i] = w[i];
      q.cs = 3.0 / 2.0;
      q.order = 7;
      break;
    }
    case Q_D2Q37: {  // src/quadratures/D2Q37.jl:11-74
      set_c(q, {0, 1, -1, 0, 0, 1, -1, 1, -1, 2, -2, 0, 0, 2, -2, -2, 2, 1, -1, 1, -1, 2, -2, 2, -2,
                3, -3, 0, 0, 3, -3, 3, -3, 1, -1, -1, 1},
            {0, 0, 0, 1, -1, 1, -1, -1, 1, 0, 0, 2, -2, 1, -1, 1, -1, 2, -2, -2, 2, 2, -2, -2, 2,
             0, 0, 3, -3, 1, -1, -1, 1, 3, -3, 3, -3});
      const double g1 = 0.23315066913235250228650, g2 = 0.10730609154221900241246,
                   g3 = 0.05766785988879488203006, g4 = 0.01420821615845075026469,
                   g5 = 0.00535304900051377523273, g6 = 0.00101193759267357547541,
                   g7 = 0.00024530102775771734547, g8 = 0.00028341425299419821740;
      int i = 0;
      q.w[i++] = g1;
      for (int k = 0; k < 4; ++k) q.w[i++] = g2;
      for (int k = 0; k < 4; ++k) q.w[i++] = g3;
      for (int k = 0; k < 4; ++k) q.w[i++] = g4;
      for (int k = 0; k < 8; ++k) q.w[i++] = g5;
      for (int k = 0; k < 4; ++k) q.w[i++] = g6;
      for (int k = 0; k < 4; ++k) q.w[i++] = g7;
      for (int k = 0; k < 8; ++k) q.w[i++] = g8;
      const double r = 1.19697977039307435897239;
      q.cs = r * r;
      q.order = 9;
      break;
    }
  }
  return q;
}

// opposite(q, idx): src/quadratures.jl:11-19 (generic), D2Q4.jl:26-31, D2Q5.jl:34-42,
// D2Q9.jl:30-38.  0-based here.
static int opposite(const Quad& q, int j) {
  const int idx = j + 1;
  int r;
  switch (q.id) {
    case Q_D2Q4: r = idx <= 2 ? idx + 2 : idx - 2; break;
    case Q_D2Q5: r = idx == 1 ? 1 : (idx <= 3 ? idx + 2 : idx - 2); break;
    case Q_D2Q9: r = idx == 1 ? 1 : (idx <= 5 ? idx + 4 : idx - 4); break;
    default: r = idx == 1 ? 1 : ((idx % 2 == 0) ? idx + 1 : idx - 1); break;
  }
  return r - 1;
}

// ---------------------------------------------------------------------------------------
// L1: Hermite tensors and equilibria
// ---------------------------------------------------------------------------------------
static inline int dlt(int a, int b) { return a == b ? 1 : 0; }

// Forward-mode dual number v + d ε (ε² = 0).  Instantiating the equilibrium, moment, SRT/TRT
// collision and stream templates below with it carries one directional derivative alongside
// every value: the forward-mode stand-in for ForwardDiff through the reference loop (the
// reference itself cannot take dual numbers: srt.jl:2 types τ as Float64).  The value part
// repeats the double arithmetic operation for operation, so it equals the double loop bitwise.
struct Dual {
  double v = 0.0, d = 0.0;
  Dual() = default;
  Dual(double a) : v(a) {}
  Dual(double a, double b) : v(a), d(b) {}
};
inline Dual operator+(Dual a, Dual b) { return {a.v + b.v, a.d + b.d}; }
inline Dual operator-(Dual a, Dual b) { return {a.v - b.v, a.d - b.d}; }
inline Dual operator-(Dual a) { return {-a.v, -a.d}; }
inline Dual operator*(Dual a, Dual b) { return {a.v * b.v, a.d * b.v + a.v * b.d}; }
inline Dual operator/(Dual a, Dual b) {
  const double q = a.v / b.v;
  return {q, (a.d - q * b.d) / b.v};
}
inline Dual& operator+=(Dual& a, Dual b) { return a = a + b; }

// hermite(Val{n}, ξ, q): src/hermite_polynomials.jl:47-82.  Tensors are flattened
// column-major (first index fastest), 2^n entries.  cs = 1 / q.speed_of_sound_squared.
static void hermite_q(int n, const int* xi, double cs, double* H) {
  if (n == 1) {
    H[0] = xi[0] * 1.0;
    H[1] = xi[1] * 1.0;
  } else if (n == 2) {
    for (int b = 0; b < 2; ++b)
      for (int a = 0; a < 2; ++a) H[a + 2 * b] = (double)(xi[b] * xi[a]) - cs * dlt(a, b);
  } else if (n == 3) {
    for (int c = 0; c < 2; ++c)
      for (int b = 0; b < 2; ++b)
        for (int a = 0; a < 2; ++a)
          H[a + 2 * b + 4 * c] = (double)(xi[c] * xi[b] * xi[a]) -
                                 cs * (double)(xi[a] * dlt(b, c) + xi[b] * dlt(a, c) + xi[c] * dlt(a, b));
  } else if (n == 4) {
    for (int e = 0; e < 2; ++e)
      for (int c = 0; c < 2; ++c)
        for (int b = 0; b < 2; ++b)
          for (int a = 0; a < 2; ++a)
            H[a + 2 * b + 4 * c + 8 * e] =
                (double)(xi[e] * xi[c] * xi[b] * xi[a]) -
                cs * (double)(xi[a] * xi[b] * dlt(c, e) + xi[a] * xi[c] * dlt(b, e) +
                              xi[a] * xi[e] * dlt(b, c) + xi[b] * xi[c] * dlt(a, e) +
                              xi[b] * xi[e] * dlt(a, c) + xi[c] * xi[e] * dlt(a, b)) +
                (cs * cs) * (double)(dlt(a, b) * dlt(c, e) + dlt(a, c) * dlt(b, e) + dlt(a, e) * dlt(b, c));
  }
}

// equilibrium_coefficient(Val{n}, q, ρ, u, T): src/velocity_distribution_function/hermite.jl:37-77
// (including the repeated δ(b,d) / δ(a,d) terms of the n = 4 case).
static void eq_coeff(int n, double cs_inv_field, double rho, const double* u, double T, double* A) {
  const double cs = 1.0 / cs_inv_field;
  if (n == 1) {
    A[0] = rho * u[0];
    A[1] = rho * u[1];
  } else if (n == 2) {
    const double lam = cs * (T - 1.0);
    for (int b = 0; b < 2; ++b)
      for (int a = 0; a < 2; ++a) {
        double m = u[a] * u[b];
        if (a == b) m = m + lam;
        A[a + 2 * b] = rho * m;
      }
  } else if (n == 3) {
    const double lam = cs * (T - 1.0);
    for (int c = 0; c < 2; ++c)
      for (int b = 0; b < 2; ++b)
        for (int a = 0; a < 2; ++a)
          A[a + 2 * b + 4 * c] =
              rho * (u[a] * u[b] * u[c] +
                     lam * ((u[a] * dlt(b, c) + u[b] * dlt(a, c)) + u[c] * dlt(a, b)));
  } else if (n == 4) {
    const double lam = cs * (T - 1.0);
    const double lam2 = (cs * cs) * ((T - 1.0) * (T - 1.0));
    for (int d = 0; d < 2; ++d)
      for (int c = 0; c < 2; ++c)
        for (int b = 0; b < 2; ++b)
          for (int a = 0; a < 2; ++a)
            A[a + 2 * b + 4 * c + 8 * d] =
                rho * (u[a] * u[b] * u[c] * u[d] +
                       lam * (u[a] * u[b] * dlt(c, d) + u[a] * u[c] * dlt(b, d) +
                              u[a] * u[d] * dlt(b, d) + u[b] * u[c] * dlt(a, d) +
                              u[b] * u[d] * dlt(a, d) + u[c] * u[d] * dlt(a, b)) +
                       lam2 * (double)(dlt(a, b) * dlt(c, d) + dlt(a, c) * dlt(b, d) + dlt(a, d) * dlt(b, c)));
  }
}

static double dot_arr(const double* a, const double* b, int m) {
  double s = 0.0;
  for (int k = 0; k < m; ++k) s += a[k] * b[k];
  return s;
}

static double factorial(int n) {
  double r = 1;
  for (int k = 2; k <= n; ++k) r *= k;
  return r;
}

// hermite_based_equilibrium!: src/velocity_distribution_function/hermite.jl:10-33.
// Used by `equilibrium(q, ρ, u, T)` (maxwell_boltzmann_equilibrium.jl:1-10), i.e. by the
// initial conditions.
static void hermite_equilibrium(const Quad& q, double rho, const double* u, double T, double* f) {
  const int N = q.order / 2;
  const double cs = 1.0 / q.cs;
  double aeq[5][16];
  for (int n = 1; n <= N; ++n) eq_coeff(n, q.cs, rho, u, T, aeq[n]);
  for (int i = 0; i < q.Q; ++i) {
    const int xi[2] = {q.cx[i], q.cy[i]};
    double s = 0.0;
    for (int n = 1; n <= N; ++n) {
      double H[16];
      hermite_q(n, xi, cs, H);
      const double term = dot_arr(aeq[n], H, 1 << n) / (factorial(n) * std::pow(cs, n));
      s = (n == 1) ? term : s + term;
    }
    f[i] = q.w[i] * (rho + s);
  }
}

// `equilibrium!` used by the collision operators:
//   generic second-order form       maxwell_boltzmann_equilibrium.jl:12-66
//   third order for D2Q17 / D2Q21   velocity_distribution_function/quadratures.jl:3-19,45-61
//   fourth order for D2Q37          velocity_distribution_function/quadratures.jl:63-124
//   first order for D2Q4 / D2Q5     velocity_distribution_function/quadratures.jl:129-159
template <class R>
static void equilibrium(const Quad& q, R rho, const R* u, R* f) {
  R u_squared = 0.0;
  for (int d = 0; d < 2; ++d) u_squared += u[d] * u[d];
  const double cs = q.cs;
  for (int i = 0; i < q.Q; ++i) {
    const R cu = q.cx[i] * u[0] + q.cy[i] * u[1];
    const R rw = rho * q.w[i];
    const R a1 = cs * cu;
    switch (q.id) {
      case Q_D2Q4:
      case Q_D2Q5:
        f[i] = rw * (1.0 + a1);
        break;
      case Q_D2Q9:
      case Q_D2Q13: {
        const R a2 = ((cs * cs) * (cu * cu) + 0.0) + (-cs * u_squared);
        f[i] = rw * ((1.0 + a1) + 0.5 * a2);
        break;
      }
      case Q_D2Q17:
      case Q_D2Q21: {
        const R a2 = ((cs * cs) * (cu * cu) + 0.0) + (-cs * u_squared);
        const R a3 = (cs * cu) * (((cs * cs) * (cu * cu) - (3.0 * cs) * u_squared) + 0.0);
        f[i] = rw * (((1.0 + a1) + 0.5 * a2) + (1.0 / 6.0) * a3);
        break;
      }
      case Q_D2Q37: {
        const R a2 = ((cs * cs) * (cu * cu) + 0.0) + (-cs * u_squared);
        const R a3 = (cs * cu) * (((cs * cs) * (cu * cu) - (3.0 * cs) * u_squared) + 0.0);
        const double cs2 = cs * cs, cs3 = cs2 * cs, cs4 = cs2 * cs2;
        const R cu2 = cu * cu;
        const R a4 = (cs4 * (cu2 * cu2) - ((6.0 * cs3) * u_squared) * cu2) +
                     (3.0 * cs2) * (u_squared * u_squared);
        f[i] = rw * ((((1.0 + a1) + 0.5 * a2) + (1.0 / 6.0) * a3) + (1.0 / 24.0) * a4);
        break;
      }
    }
  }
}

// density / velocity!: src/velocity_distribution_function/moments.jl:1-19
template <class R>
static R density(const Quad& q, const R* f) {
  R s = f[0];
  for (int i = 1; i < q.Q; ++i) s += f[i];
  return s;
}
template <class R>
static void velocity(const Quad& q, const R* f, R rho, R* u) {
  for (int d = 0; d < 2; ++d) {
    R s = 0.0;
    const int* c = d == 0 ? q.cx : q.cy;
    for (int i = 0; i < q.Q; ++i) s += f[i] * c[i];
    u[d] = s / rho;
  }
}
// a_bar_2 = Σ_i f_i H_2(c_i) with H_2 from hermite(Val{2}, ξ, q)
static void second_moment(const Quad& q, const double* f, double* a2) {
  const double cs = 1.0 / q.cs;
  for (int k = 0; k < 4; ++k) a2[k] = 0.0;
  for (int i = 0; i < q.Q; ++i) {
    const int xi[2] = {q.cx[i], q.cy[i]};
    double H[4];
    hermite_q(2, xi, cs, H);
    for (int k = 0; k < 4; ++k) a2[k] = (i == 0) ? f[i] * H[k] : a2[k] + f[i] * H[k];
  }
}
// pressure(q, f, ρ, u): moments.jl:21-33; D2Q4 / D2Q5 overrides (quadratures.jl:125-127, D2Q5.jl:43)
static double pressure(const Quad& q, const double* f, double rho, const double* u) {
  if (q.id == Q_D2Q4 || q.id == Q_D2Q5) return 1.0;
  double a2[4];
  second_moment(q, f, a2);
  return ((a2[0] + a2[3]) - rho * ((u[0] * u[0] + u[1] * u[1]) - 2.0)) / 2.0;
}
// deviatoric_tensor(q, τ, f, ρ, u): moments.jl:81-96
static void deviatoric_tensor(const Quad& q, double tau, const double* f, double rho,
                              const double* u, double* sigma) {
  double a2[4], aeq[4];
  second_moment(q, f, a2);
  eq_coeff(2, q.cs, rho, u, 1.0, aeq);
  double s[4];
  const double den = 1.0 + 1.0 / (2.0 * tau);
  for (int k = 0; k < 4; ++k) s[k] = (a2[k] - aeq[k]) / den;
  const double tr = (s[0] + s[3]) / 2.0;
  sigma[0] = s[0] - tr;
  sigma[1] = s[1];
  sigma[2] = s[2];
  sigma[3] = s[3] - tr;
}

// ---------------------------------------------------------------------------------------
// L3: problems (src/problems/*.jl) -- analytic fields, forces, unit conversion
// ---------------------------------------------------------------------------------------
enum ProblemKind {
  P_TAYLOR_GREEN = 0,  // TaylorGreenVortex  taylor_green_vortex.jl
  P_TGV = 1,           // TGV                second_order_convergence.jl
  P_POISEUILLE = 2,    // PoiseuilleFlow     poiseuille.jl
  P_COUETTE = 3,       // CouetteFlow        couette_flow.jl
  P_DECAYING_SHEAR = 4,// DecayingShearFlow  decaying_shear_flow.jl
  P_LID_DRIVEN = 5,    // LidDrivenCavityFlow lid_driven_cavity.jl
  P_LIN_THERMAL = 6,   // LinearizedThermalDiffusion linear_hydrodynamics_modes.jl
  P_LIN_SHEAR = 7,     // LinearizedTransverseShearWave linear_hydrodynamics_modes.jl
  P_INIT_TEST = 8,     // InitializationTestProblem (test/initial_conditions.jl:12-87)
  P_SHEAR_WAVE = 9,    // lattice-unit shear wave u_x = u0 sin(2π y / Ny) (user problem type)
};

}  // namespace orc

extern "C" {
// Flat problem description shared with the Python wrapper (oracle/oracle.py).
typedef struct {
  int kind, nx, ny, is_static;
  double rho_0, u_max, nu, dom0, dom1;
  double A, B, a, b;    // TaylorGreenVortex A,B,a,b ; DecayingShearFlow A,B
  double k_x, k_y;      // DecayingShearFlow
  double G, k;          // PoiseuilleFlow
  double u_0, tau;      // TGV
  double theta_0, rho_t, u_t, kappa;  // Linearized* modes
  double q_cs;          // TGV: speed_of_sound_squared of the quadrature it was built with
} orc_problem;
}

namespace orc {

struct Vec2 { double x, y; };
struct Mat2 { double m[4]; };  // column-major [a11 a21 a12 a22]

static double delta_x(const orc_problem& p) {
  switch (p.kind) {
    case P_TGV: case P_SHEAR_WAVE: return 1.0;                           // second_order_convergence.jl:120
    case P_POISEUILLE: return p.dom1 / p.ny;                             // poiseuille.jl:84-86
    case P_LIN_THERMAL: case P_LIN_SHEAR: return p.dom1 / p.ny;          // linear_hydrodynamics_modes.jl:56,144
    default:                                                             // problems.jl:89-95
      if (p.nx > p.ny) return p.dom0 * (1.0 / p.nx);
      return p.dom1 * (1.0 / p.ny);
  }
}
static double delta_t(const orc_problem& p) {
  if (p.kind == P_TGV || p.kind == P_SHEAR_WAVE) return 1.0;  // second_order_convergence.jl:121
  return delta_x(p) * p.u_max;                                // problems.jl:85-87
}
static double viscosity(const orc_problem& p) {
  if (p.kind == P_TGV || p.kind == P_SHEAR_WAVE) return p.nu;  // second_order_convergence.jl:119
  const double dx = delta_x(p);
  return p.nu * (dx * dx) / delta_t(p);  // problems.jl:80
}
static double heat_diffusion(const orc_problem& p) {
  const double dx = delta_x(p);
  return p.kappa * (dx * dx) / delta_t(p);  // problems.jl:81-82
}
static double tgv_td(const orc_problem& p, double* kx, double* ky) {
  *kx = 2 * M_PI / p.nx;
  *ky = 2 * M_PI / p.ny;
  return 1.0 / (p.nu * ((*kx) * (*kx) + (*ky) * (*ky)));
}

static double decay(const orc_problem& p, double x, double y, double t) {
  (void)x; (void)y;
  if (p.kind == P_TAYLOR_GREEN)  // taylor_green_vortex.jl:106-111
    return p.is_static ? 1.0 : std::exp(-(p.a * p.a + p.b * p.b) * viscosity(p) * t);
  if (p.kind == P_DECAYING_SHEAR)  // decaying_shear_flow.jl:118-131
    return p.is_static ? 1.0 : std::exp(-1.0 * (p.k_x * p.k_x) * viscosity(p) * t);
  if (p.kind == P_TGV) {
    double kx, ky;
    const double td = tgv_td(p, &kx, &ky);
    return p.is_static ? 1.0 : std::exp(-t / td);
  }
  return 1.0;
}

static double pressure_a(const orc_problem& p, double cs_field, double x, double y, double t) {
  switch (p.kind) {
    case P_TAYLOR_GREEN: {  // taylor_green_vortex.jl:49-69
      const double d = decay(p, x, y, t);
      const double P = -(1.0 / 4.0) * p.rho_0 * (d * d) *
                       ((p.A * p.A) * std::cos(2 * p.a * x) + (p.B * p.B) * std::cos(2 * p.b * y));
      return 1.0 + cs_field * (p.u_max * p.u_max) * P;
    }
    case P_TGV: {  // second_order_convergence.jl:47-66
      double kx, ky;
      const double td = tgv_td(p, &kx, &ky);
      const double X = x * p.nx, Y = y * p.ny;
      const double p0 = p.rho_0, rho = 1.0;
      return p0 - cs_field * rho * ((p.u_0 * p.u_0) / 4) *
                      ((ky / kx) * std::cos(2 * kx * X) + (kx / ky) * std::cos(2 * ky * Y)) *
                      std::exp(-2 * t / td);
    }
    case P_DECAYING_SHEAR: {  // decaying_shear_flow.jl:50-74
      const double s = std::sin(p.k_x * (x - p.A * t));
      const double d = decay(p, x, y, t);
      return 1 + p.B * (0.025) * cs_field * (p.u_max * p.u_max) * p.B * (s * s) * (d * d);
    }
    case P_LIN_THERMAL: return p.rho_0 * p.theta_0;
    case P_LIN_SHEAR: return p.theta_0;
    case P_INIT_TEST:  // test/initial_conditions.jl:37-46 (U = 0.001)
      return 1.0 - (1.0 / 4.0) * cs_field * (p.u_max * p.u_max) * (0.001 * 0.001) *
                       (std::cos(2 * x) + std::cos(2 * y));
    default: return 1.0;
  }
}

static double density_a(const orc_problem& p, double cs_field, double x, double y, double t) {
  switch (p.kind) {
    case P_TAYLOR_GREEN: return pressure_a(p, cs_field, x, y, t);  // taylor_green_vortex.jl:37-48
    case P_TGV: {  // second_order_convergence.jl:28-46
      double kx, ky;
      const double td = tgv_td(p, &kx, &ky);
      const double X = x * p.nx, Y = y * p.ny;
      return p.rho_0 * (1.0 - cs_field * ((p.u_0 * p.u_0) / 4) *
                                  ((ky / kx) * std::cos(2 * kx * X) + (kx / ky) * std::cos(2 * ky * Y)) *
                                  std::exp(-2 * t / td));
    }
    case P_LIN_THERMAL:
      return p.rho_0 + p.rho_t * std::sin(y) * std::exp(-heat_diffusion(p) * t);
    case P_LIN_SHEAR: return p.rho_0;
    case P_INIT_TEST: return pressure_a(p, cs_field, x, y, t);
    default: return 1.0;
  }
}

static Vec2 velocity_a(const orc_problem& p, double x, double y, double t) {
  switch (p.kind) {
    case P_TAYLOR_GREEN: {  // taylor_green_vortex.jl:71-85
      const double d = decay(p, x, y, t);
      return {d * (p.A * std::cos(p.a * x) * std::sin(p.b * y)),
              d * (p.B * std::sin(p.a * x) * std::cos(p.b * y))};
    }
    case P_TGV: {  // second_order_convergence.jl:68-84
      double kx, ky;
      const double td = tgv_td(p, &kx, &ky);
      const double X = x * p.nx, Y = y * p.ny;
      const double s = p.u_0 * std::exp(-t / td);
      return {s * (-std::sqrt(ky / kx) * std::cos(kx * X) * std::sin(ky * Y)),
              s * (std::sqrt(kx / ky) * std::sin(kx * X) * std::cos(ky * Y))};
    }
    case P_POISEUILLE:  // poiseuille.jl:48-58
      return {y * (p.dom1 - y) * (p.G / 2), 0.0};
    case P_COUETTE: return {y, 0.0};  // couette_flow.jl:47-52
    case P_DECAYING_SHEAR: {  // decaying_shear_flow.jl:76-93
      if (p.is_static)
        return {p.A * std::cos(p.k_y * y - p.k_y * p.B * t), p.B * std::cos(p.k_x * x - p.k_x * p.A * t)};
      const double nu = viscosity(p);
      return {p.A * std::cos(p.k_y * y - p.k_y * p.B * t) * std::exp(-1.0 * (p.k_y * p.k_y) * nu * t),
              p.B * std::cos(p.k_x * x - p.k_x * p.A * t) * std::exp(-1.0 * (p.k_x * p.k_x) * nu * t)};
    }
    case P_LIN_SHEAR:  // linear_hydrodynamics_modes.jl:168-177
      return {p.u_t * std::sin(y) * std::exp(-viscosity(p) * t), 0.0};
    case P_INIT_TEST: {  // test/initial_conditions.jl:47-56
      const double s = p.u_max * 0.001;
      return {s * (std::cos(2 * M_PI * x) * std::sin(2 * M_PI * y)),
              s * (-std::sin(2 * M_PI * x) * std::cos(2 * M_PI * y))};
    }
    case P_SHEAR_WAVE: {
      const double k = 2 * M_PI / p.ny;
      return {p.u_0 * std::sin(k * y) * std::exp(-p.nu * (k * k) * t), 0.0};
    }
    default: return {0.0, 0.0};
  }
}

// velocity_gradient: the matrix [u_x v_x; u_y v_y] (row-major as written in Julia), stored
// column-major: m = [u_x, u_y, v_x, v_y].
static Mat2 velocity_gradient(const orc_problem& p, double x, double y, double t) {
  Mat2 g{{0, 0, 0, 0}};
  double ux = 0, vy = 0, uy = 0, vx = 0, s = 1.0;
  switch (p.kind) {
    case P_TAYLOR_GREEN:  // taylor_green_vortex.jl:87-104
      ux = -p.a * p.A * std::sin(p.a * x) * std::sin(p.b * y);
      vy = -p.b * p.B * std::sin(p.a * x) * std::sin(p.b * y);
      uy = p.b * p.A * std::cos(p.a * x) * std::cos(p.b * y);
      vx = p.a * p.B * std::cos(p.a * x) * std::cos(p.b * y);
      s = decay(p, x, y, t);
      break;
    case P_TGV: {  // second_order_convergence.jl:86-103
      double kx, ky;
      const double td = tgv_td(p, &kx, &ky);
      const double X = x * p.nx, Y = y * p.ny;
      ux = std::sqrt(ky * kx) * std::sin(kx * X) * std::sin(ky * Y);
      vy = -std::sqrt(ky * kx) * std::sin(kx * X) * std::sin(ky * Y);
      uy = -std::sqrt((ky * ky * ky) / kx) * std::cos(kx * X) * std::cos(ky * Y);
      vx = std::sqrt((kx * kx * kx) / ky) * std::cos(kx * X) * std::cos(ky * Y);
      s = std::exp(-t / td) * p.u_0;
      break;
    }
    case P_POISEUILLE:  // poiseuille.jl:59-71
      uy = (p.dom1 - 2 * y) * (p.G / 2);
      break;
    case P_COUETTE: uy = 1.0; break;  // couette_flow.jl:53-66
    case P_DECAYING_SHEAR: {  // decaying_shear_flow.jl:95-116
      uy = -p.A * p.k_y * std::sin(p.k_y * (y - p.B * t));
      vx = -p.B * p.k_x * std::sin(p.k_x * (x - p.A * t));
      if (!p.is_static) {
        const double nu = viscosity(p);
        uy *= std::exp(-1.0 * (p.k_y * p.k_y) * nu * t);
        vx *= std::exp(-1.0 * (p.k_x * p.k_x) * nu * t);
      }
      break;
    }
    case P_INIT_TEST: {  // test/initial_conditions.jl:57-69
      ux = -std::sin(2 * M_PI * x) * std::sin(2 * M_PI * y);
      vy = std::sin(2 * M_PI * x) * std::sin(2 * M_PI * y);
      uy = std::cos(2 * M_PI * x) * std::cos(2 * M_PI * y);
      vx = -std::cos(2 * M_PI * x) * std::cos(2 * M_PI * y);
      s = p.u_max * 0.001 * 2 * M_PI;
      break;
    }
    case P_SHEAR_WAVE: {
      const double k = 2 * M_PI / p.ny;
      uy = p.u_0 * k * std::cos(k * y) * std::exp(-p.nu * (k * k) * t);
      break;
    }
    default: break;
  }
  g.m[0] = s * ux;
  g.m[1] = s * uy;
  g.m[2] = s * vx;
  g.m[3] = s * vy;
  return g;
}

// deviatoric_tensor(q, problem, x, y, t): problems.jl:30-46 (test problem: ×NX,
// test/initial_conditions.jl:71-87).  Returned column-major [σxx σyx σxy σyy].
static Mat2 deviatoric_a(const orc_problem& p, double x, double y, double t) {
  const Mat2 a = velocity_gradient(p, x, y, t);
  const double nu = viscosity(p);
  const double a11 = a.m[0], a21 = a.m[1], a12 = a.m[2], a22 = a.m[3];
  Mat2 s;
  s.m[0] = -nu * (2 * a11);
  s.m[1] = -nu * (a12 + a21);
  s.m[2] = -nu * (a12 + a21);
  s.m[3] = -nu * (2 * a22);
  if (p.kind == P_INIT_TEST)
    for (int k = 0; k < 4; ++k) s.m[k] = s.m[k] * p.nx;
  return s;
}

// force(problem, x, y, t) before lattice scaling.
static Vec2 force_a(const orc_problem& p, double x, double y, double t) {
  switch (p.kind) {
    case P_TAYLOR_GREEN:  // taylor_green_vortex.jl:113-116
      if (p.is_static) {
        const Vec2 v = velocity_a(p, x, y, 0.0);
        const double s = 2 * viscosity(p);
        return {s * v.x, s * v.y};
      }
      return {0, 0};
    case P_TGV:  // second_order_convergence.jl:105-109
      if (p.is_static) {
        const Vec2 v = velocity_a(p, x, y, 0.0);
        return {2 * p.nu * v.x, 2 * p.nu * v.y};
      }
      return {0, 0};
    case P_POISEUILLE: return {viscosity(p) * p.G, 0.0};  // poiseuille.jl:72-82
    case P_DECAYING_SHEAR:  // decaying_shear_flow.jl:132-147
      if (!p.is_static) return {0, 0};
      return {viscosity(p) * (p.k_y * p.k_y) * p.A * std::cos(p.k_y * y - p.k_y * p.B * t),
              viscosity(p) * (p.k_x * p.k_x) * p.B * std::cos(p.k_x * x - p.k_x * p.A * t)};
    default: return {0, 0};
  }
}
static bool has_external_force(const orc_problem& p) {
  switch (p.kind) {
    case P_TAYLOR_GREEN: case P_TGV: case P_DECAYING_SHEAR: return p.is_static != 0;
    case P_POISEUILLE: return true;
    default: return false;
  }
}

// range(problem): problems.jl:18-26 -- Julia's range(a, stop=b, length=n) evaluated in
// extended precision then rounded (Julia uses TwicePrecision for Float64 ranges).  The y
// range uses domain_size[1] for its stop, as the reference does.
static void make_range(double a, double b, int n, std::vector<double>& out, double* step) {
  out.resize(n);
  if (n == 1) {
    out[0] = a;
    *step = 0.0;  // Julia: a length-1 range has step start - stop = 0
    return;
  }
  const long double st = ((long double)b - (long double)a) / (long double)(n - 1);
  for (int i = 0; i < n; ++i) out[i] = (double)((long double)a + st * (long double)i);
  *step = (double)st;
}
static void ranges(const orc_problem& p, std::vector<double>& xr, std::vector<double>& yr,
                   double* xstep, double* ystep) {
  const double dx = p.dom0 / p.nx, dy = p.dom1 / p.ny;
  make_range(dx / 2, p.dom0 - dx / 2, p.nx, xr, xstep);
  make_range(dy / 2, p.dom0 - dy / 2, p.ny, yr, ystep);
}

static Vec2 lattice_velocity(const orc_problem& p, double x, double y) {
  const Vec2 v = velocity_a(p, x, y, 0.0);  // problems.jl:99-100
  return {p.u_max * v.x, p.u_max * v.y};
}

}  // namespace orc

// ---------------------------------------------------------------------------------------
// Collision models, BCs, model, processing (L2, L4, L5)
// ---------------------------------------------------------------------------------------
extern "C" {
typedef struct {
  int kind;        // 0 SRT, 1 TRT, 2 MRT, 3 iterative-initialisation (Mei et al.)
  double tau[8];   // SRT: τ ; TRT: τ_s, τ_a ; MRT: τs[1..n] ; iterative: τ
  int ntau;
  int force_kind;  // 0 none, 1 the problem's lattice_force closure
} orc_collision;

typedef struct {
  int kind;        // 0 BounceBack, 1 MovingWall
  int direction;   // 0 North, 1 East, 2 South, 3 West
  int x_lo, x_hi, y_lo, y_hi;  // 1-based inclusive ranges (xs, ys)
  double u[2], rho, T;
} orc_bc;
}

namespace orc {

struct Model {
  Quad q;
  orc_problem prob;
  orc_collision cm;
  std::vector<orc_bc> bcs;
  int nx, ny;
  std::vector<double> f_stream, f_collision;
  std::vector<double> nonlinear;  // iterative-initialisation collision (iterative_initialization.jl:12-40)
  std::vector<double> xr, yr;
  double xstep = 0, ystep = 0;
  int nthreads = 1;
  size_t idx(int x, int y, int i) const { return (size_t)x + (size_t)nx * ((size_t)y + (size_t)ny * i); }
};

static Vec2 lattice_force(const Model& m, int xi, int yi, double t) {
  // lattice_force(problem, x_idx, y_idx, t): problems.jl:62-74,103-104; integer-index
  // specialisations for Poiseuille / Couette (poiseuille.jl:72, couette_flow.jl:67).
  const orc_problem& p = m.prob;
  const Vec2 F = force_a(p, m.xr[xi], m.yr[yi], t);
  const double s = p.u_max * delta_t(p);
  return {s * F.x, s * F.y};
}

// One node of collide! for SRT (srt.jl:18-62, kind 0, τ = tau0) and TRT (trt.jl:42-97,
// kind 1, τ_s = tau0, τ_a = tau1): f holds the node's Q populations, (Fx, Fy) its lattice force
// (added to u times τ, resp. τ_a, when `force`), out receives the post-collision populations.
template <class R>
static void collide_srt_trt_node(const Quad& q, int kind, R tau0, R tau1, bool force, R Fx, R Fy, const R* f,
                                 R* out) {
  const int Q = q.Q;
  const R rho = density(q, f);
  R u[2], feq[37];
  velocity(q, f, rho, u);
  const R shift = kind == 0 ? tau0 : tau1;
  if (force) {
    const R us[2] = {u[0] + shift * Fx, u[1] + shift * Fy};
    equilibrium(q, rho, us, feq);
  } else {
    equilibrium(q, rho, (const R*)u, feq);
  }
  if (kind == 0) {
    const R tau = tau0;
    for (int i = 0; i < Q; ++i) out[i] = (1 - 1 / tau) * f[i] + (1 / tau) * feq[i];
  } else {
    const R ts = tau0, ta = tau1;
    for (int i = 0; i < Q; ++i) {
      const int o = opposite(q, i);
      const R feq_s = 0.5 * (feq[i] + feq[o]);
      const R feq_a = 0.5 * (feq[i] - feq[o]);
      const R f_s = 0.5 * (f[i] + f[o]);
      const R f_a = 0.5 * (f[i] - f[o]);
      out[i] = f[i] + (-(1 / ts) * (f_s - feq_s) - (1 / ta) * (f_a - feq_a));
    }
  }
}

// One node of the MRT collide! of a second-order set (mrt.jl:56-118 with N = div(order, 2) = 2:
// D2Q9, D2Q13) for any number type R, operation for operation the double path of collide()
// below: tau1, tau2 are τs[1], τs[2]; the force shift uses τs[2] (mrt.jl:91-95); the first-order
// coefficient a_coll[1] is formed there but never used, so it is skipped.  Hs: the Hermite tables
// of collide() (mrt.jl:29-34).
template <class R>
static void collide_mrt2_node(const Quad& q, const double (*Hs)[37][16], R tau1, R tau2, bool force, R Fx, R Fy,
                              const R* f, R* out) {
  (void)tau1;
  const int Q = q.Q;
  const double cs = q.cs;
  const R rho = density(q, f);
  R u[2];
  velocity(q, f, rho, u);
  if (force) {
    u[0] = u[0] + tau2 * Fx;
    u[1] = u[1] + tau2 * Fy;
  }
  R aeq[4], af[4], acoll[4];
  for (int b = 0; b < 2; ++b)  // equilibrium_coefficient(Val{2}, q, ρ, u, T = 1): hermite.jl:37-77
    for (int a = 0; a < 2; ++a) {
      R m = u[a] * u[b];
      if (a == b) m = m + 0.0;
      aeq[a + 2 * b] = rho * m;
    }
  for (int k = 0; k < 4; ++k) {
    R sm = f[0] * Hs[2][0][k];
    for (int i = 1; i < Q; ++i) sm = sm + f[i] * Hs[2][i][k];
    af[k] = sm;
  }
  for (int k = 0; k < 4; ++k) acoll[k] = (1 - 1 / tau2) * af[k] + (1 / tau2) * aeq[k];
  for (int i = 0; i < Q; ++i) {
    const R first = cs * rho * (u[0] * Hs[1][i][0] + u[1] * Hs[1][i][1]);
    R dot = 0.0;
    for (int k = 0; k < 4; ++k) dot += acoll[k] * Hs[2][i][k];
    const R hi = std::pow(cs, 2) * dot / factorial(2);
    out[i] = q.w[i] * ((rho + first) + hi);
  }
}

// collide! for SRT (srt.jl:18-62), TRT (trt.jl:42-97), MRT (mrt.jl:49-118), and the
// iterative-initialisation model (iterative_initialization.jl:41-60).  Loop order x outer,
// y inner, as in the reference.
static void collide(Model& m, const std::vector<double>& fin, std::vector<double>& fout, double time) {
  const Quad& q = m.q;
  const int Q = q.Q;
  const int nx = m.nx, ny = m.ny;
  const orc_collision& cm = m.cm;
  const int N = q.order / 2;
  const double csinv = 1.0 / q.cs;
  // MRT Hermite tables (mrt.jl:29-34)
  double Hs[5][37][16];
  if (cm.kind == 2)
    for (int n = 1; n <= N; ++n)
      for (int i = 0; i < Q; ++i) {
        const int xi[2] = {q.cx[i], q.cy[i]};
        hermite_q(n, xi, csinv, Hs[n][i]);
      }
#pragma omp parallel for schedule(static) num_threads(m.nthreads) if (m.nthreads > 1)
  for (int x = 0; x < nx; ++x) {
    double f[37];
    for (int y = 0; y < ny; ++y) {
      for (int i = 0; i < Q; ++i) f[i] = fin[m.idx(x, y, i)];
      if (cm.kind == 0 || cm.kind == 1) {  // SRT, TRT
        double Fx = 0.0, Fy = 0.0, out[37];
        if (cm.force_kind) {
          const Vec2 F = lattice_force(m, x, y, time);
          Fx = F.x;
          Fy = F.y;
        }
        collide_srt_trt_node<double>(q, cm.kind, cm.tau[0], cm.tau[1], cm.force_kind != 0, Fx, Fy, f, out);
        for (int i = 0; i < Q; ++i) fout[m.idx(x, y, i)] = out[i];
        continue;
      }
      const double rho = density(q, f);
      double u[2];
      velocity(q, f, rho, u);
      if (cm.kind == 2) {  // MRT (regularised / projected)
        const double cs = q.cs;
        if (cm.force_kind) {
          const Vec2 F = lattice_force(m, x, y, time);
          u[0] = u[0] + cm.tau[1] * F.x;
          u[1] = u[1] + cm.tau[1] * F.y;
        }
        double acoll[5][16];
        for (int n = 1; n <= N; ++n) {
          double aeq[16], af[16];
          eq_coeff(n, q.cs, rho, u, 1.0, aeq);
          const int M = 1 << n;
          for (int k = 0; k < M; ++k) {
            double s = f[0] * Hs[n][0][k];
            for (int i = 1; i < Q; ++i) s = s + f[i] * Hs[n][i][k];
            af[k] = s;
          }
          const double tn = cm.tau[n - 1];
          for (int k = 0; k < M; ++k) acoll[n][k] = (1 - 1 / tn) * af[k] + (1 / tn) * aeq[k];
        }
        for (int i = 0; i < Q; ++i) {
          const double first = cs * rho * (u[0] * Hs[1][i][0] + u[1] * Hs[1][i][1]);
          double hi = 0.0;
          for (int n = 2; n <= N; ++n) {
            const double term = std::pow(cs, n) * dot_arr(acoll[n], Hs[n][i], 1 << n) / factorial(n);
            hi = (n == 2) ? term : hi + term;
          }
          fout[m.idx(x, y, i)] = q.w[i] * ((rho + first) + hi);
        }
      } else {  // iterative initialisation (Mei et al.)
        const double tau = cm.tau[0];
        for (int i = 0; i < Q; ++i) {
          const double fe = q.w[i] * rho + m.nonlinear[m.idx(x, y, i)];
          fout[m.idx(x, y, i)] = (1 - 1 / tau) * f[i] + (1 / tau) * fe;
        }
      }
    }
  }
}

static inline int mod1(int a, int n) {  // Julia mod1 for positive n, 1-based result
  int r = a % n;
  if (r <= 0) r += n;
  return r;
}

// stream!: periodic pull, stream.jl:18-30,69-74
template <class R>
static void stream_periodic(const Quad& q, int nx, int ny, const R* f, R* fnew, int nthreads) {
  auto idx = [&](int x, int y, int i) { return (size_t)x + (size_t)nx * ((size_t)y + (size_t)ny * i); };
#pragma omp parallel for schedule(static) num_threads(nthreads) if (nthreads > 1)
  for (int x = 1; x <= nx; ++x)
    for (int y = 1; y <= ny; ++y)
      for (int i = 0; i < q.Q; ++i) {
        const int fx = mod1(x - q.cx[i], nx), fy = mod1(y - q.cy[i], ny);
        fnew[idx(x - 1, y - 1, i)] = f[idx(fx - 1, fy - 1, i)];
      }
}
static void stream(Model& m, const std::vector<double>& f, std::vector<double>& fnew) {
  stream_periodic(m.q, m.nx, m.ny, f.data(), fnew.data(), m.nthreads);
}

// apply!(bcs, q, f_new, f_old): boundary_conditions.jl:6-20 in list order;
// BounceBack bounce_back.jl:8-72; MovingWall moving_wall.jl:17-38.  R is double, or the Dual of
// the forward-mode derivative (orc_tangent_loss).
template <class R>
static void apply_bcs_t(const Quad& q, int nx, int ny, const std::vector<orc_bc>& bcs, R* fnew, const R* fold) {
  auto idx = [&](int x, int y, int i) { return (size_t)x + (size_t)nx * ((size_t)y + (size_t)ny * i); };
  for (const orc_bc& bc : bcs) {
    if (bc.kind == 0) {
      for (int i = 0; i < q.Q; ++i) {
        const int o = opposite(q, i);
        if (bc.direction == 0 || bc.direction == 2) {  // North / South
          for (int y = bc.y_lo; y <= bc.y_hi; ++y) {
            const bool skip = bc.direction == 0 ? (y + q.cy[o] <= ny) : (y + q.cy[o] > 0);
            if (skip) continue;
            for (int x = bc.x_lo; x <= bc.x_hi; ++x) fnew[idx(x - 1, y - 1, i)] = fold[idx(x - 1, y - 1, o)];
          }
        } else {  // East / West
          for (int x = bc.x_lo; x <= bc.x_hi; ++x) {
            const bool skip = bc.direction == 1 ? (x + q.cx[o] <= nx) : (x + q.cx[o] > 0);
            if (skip) continue;
            for (int y = bc.y_lo; y <= bc.y_hi; ++y) fnew[idx(x - 1, y - 1, i)] = fold[idx(x - 1, y - 1, o)];
          }
        }
      }
    } else {  // MovingWall{North}: ignores xs / ys
      const double a1eq[2] = {bc.rho * bc.u[0], bc.rho * bc.u[1]};
      for (int i = 0; i < q.Q; ++i) {
        const double H1[2] = {q.cx[i] * 1.0, q.cy[i] * 1.0};
        const double a1 = q.w[i] * q.cs * (a1eq[0] * H1[0] + a1eq[1] * H1[1]);
        const int o = opposite(q, i);
        for (int y = 1; y <= ny; ++y) {
          if (y + q.cy[o] <= ny) continue;
          for (int x = 1; x <= nx; ++x) fnew[idx(x - 1, y - 1, i)] = fold[idx(x - 1, y - 1, o)] + R(2 * a1);
        }
      }
    }
  }
}
static void apply_bcs(Model& m, std::vector<double>& fnew, const std::vector<double>& fold) {
  apply_bcs_t<double>(m.q, m.nx, m.ny, m.bcs, fnew.data(), fold.data());
}

}  // namespace orc

// ---------------------------------------------------------------------------------------
// C ABI for the Python wrapper
// ---------------------------------------------------------------------------------------
using namespace orc;

extern "C" {

int orc_quadrature(int id, int* Q, int* cx, int* cy, double* w, double* cs, int* order, int* opp) {
  if (id < 0 || id > 6) return -1;
  const Quad q = make_quad(id);
  *Q = q.Q;
  *cs = q.cs;
  *order = q.order;
  for (int i = 0; i < q.Q; ++i) {
    cx[i] = q.cx[i];
    cy[i] = q.cy[i];
    w[i] = q.w[i];
    opp[i] = opposite(q, i);
  }
  return 0;
}

void orc_hermite(int qid, int n, int cx, int cy, double* H) {
  const Quad q = make_quad(qid);
  const int xi[2] = {cx, cy};
  hermite_q(n, xi, 1.0 / q.cs, H);
}

void orc_equilibrium(int qid, double rho, double ux, double uy, double* f) {
  const Quad q = make_quad(qid);
  const double u[2] = {ux, uy};
  equilibrium(q, rho, u, f);
}
void orc_hermite_equilibrium(int qid, double rho, double ux, double uy, double T, double* f) {
  const Quad q = make_quad(qid);
  const double u[2] = {ux, uy};
  hermite_equilibrium(q, rho, u, T, f);
}
void orc_moments(int qid, const double* f, double tau, double* out) {
  // out: ρ, ux, uy, pressure, temperature, σxx, σyx, σxy, σyy
  const Quad q = make_quad(qid);
  const double rho = density(q, f);
  double u[2];
  velocity(q, f, rho, u);
  const double p = pressure(q, f, rho, u);
  double s[4];
  deviatoric_tensor(q, tau, f, rho, u, s);
  out[0] = rho; out[1] = u[0]; out[2] = u[1]; out[3] = p; out[4] = p / rho;
  for (int k = 0; k < 4; ++k) out[5 + k] = s[k];
}

// Analytic fields of a problem on its lattice at time t (physical):
// out has 9 planes of nx*ny: ρ, ux, uy, p, σxx, σyx, σxy, σyy, (unused 0).
void orc_problem_fields(const orc_problem* p, int qid, double t, double* out) {
  const Quad q = make_quad(qid);
  std::vector<double> xr, yr;
  double xs, ys;
  ranges(*p, xr, yr, &xs, &ys);
  const size_t n = (size_t)p->nx * p->ny;
  for (int x = 0; x < p->nx; ++x)
    for (int y = 0; y < p->ny; ++y) {
      const size_t k = x + (size_t)p->nx * y;
      const double X = xr[x], Y = yr[y];
      out[k] = density_a(*p, q.cs, X, Y, t);
      const Vec2 v = velocity_a(*p, X, Y, t);
      out[n + k] = v.x;
      out[2 * n + k] = v.y;
      out[3 * n + k] = pressure_a(*p, q.cs, X, Y, t);
      const Mat2 s = deviatoric_a(*p, X, Y, t);
      for (int c = 0; c < 4; ++c) out[(4 + c) * n + k] = s.m[c];
      out[8 * n + k] = 0.0;
    }
}

void orc_problem_scalars(const orc_problem* p, double* out) {
  // delta_x, delta_t, viscosity, x step, y step
  std::vector<double> xr, yr;
  double xs, ys;
  ranges(*p, xr, yr, &xs, &ys);
  out[0] = delta_x(*p);
  out[1] = delta_t(*p);
  out[2] = viscosity(*p);
  out[3] = xs;
  out[4] = ys;
}

void orc_problem_coords(const orc_problem* p, double* xr_out, double* yr_out) {
  std::vector<double> xr, yr;
  double xs, ys;
  ranges(*p, xr, yr, &xs, &ys);
  for (int i = 0; i < p->nx; ++i) xr_out[i] = xr[i];
  for (int i = 0; i < p->ny; ++i) yr_out[i] = yr[i];
}

// lattice_force field (2 planes of nx*ny) at physical time t
void orc_force_field(const orc_problem* p, double t, double* out) {
  Model m;
  m.prob = *p;
  m.nx = p->nx;
  m.ny = p->ny;
  ranges(*p, m.xr, m.yr, &m.xstep, &m.ystep);
  const size_t n = (size_t)p->nx * p->ny;
  for (int x = 0; x < p->nx; ++x)
    for (int y = 0; y < p->ny; ++y) {
      const Vec2 F = lattice_force(m, x, y, t);
      out[x + (size_t)p->nx * y] = F.x;
      out[n + x + (size_t)p->nx * y] = F.y;
    }
}

// initialize(strategy, q, problem): initial_conditions.jl:7-22 and the strategies in
// initial_conditions/*.jl.  strategy: 0 ZeroVelocity, 1 AnalyticalEquilibrium,
// 2 AnalyticalEquilibriumAndOffEquilibrium, 3 ConstantDensity, 4 AnalyticalVelocityAndStress.
int orc_initialize(int strategy, int qid, const orc_problem* p, double* f) {
  const Quad q = make_quad(qid);
  std::vector<double> xr, yr;
  double xs, ys;
  ranges(*p, xr, yr, &xs, &ys);
  const int nx = p->nx, ny = p->ny, Q = q.Q;
  const double csinv = 1.0 / q.cs;
  for (int x = 0; x < nx; ++x)
    for (int y = 0; y < ny; ++y) {
      const double X = xr[x], Y = yr[y];
      double fl[37] = {0};
      if (strategy == 0) {  // initial_conditions.jl:44-53
        for (int i = 0; i < Q; ++i) fl[i] = q.w[i];
      } else if (strategy == 1 || strategy == 2) {
        const double rho = density_a(*p, q.cs, X, Y, 0.0);           // lattice_density
        const Vec2 v = lattice_velocity(*p, X, Y);                     // lattice_velocity
        const double T = pressure_a(*p, q.cs, X, Y, 0.0) / density_a(*p, q.cs, X, Y, 0.0);
        const double u[2] = {v.x, v.y};
        hermite_equilibrium(q, rho, u, T, fl);                          // problems.jl:121-128
        if (strategy == 2 && p->kind != P_TGV) {  // analytical_offequilibrium.jl:10-49
          const Mat2 g = velocity_gradient(*p, X, Y, 0.0);
          const double s2 = p->u_max * p->u_max;
          double G[4];
          for (int k = 0; k < 4; ++k) G[k] = s2 * g.m[k];
          const double S[4] = {G[0] + G[0], G[1] + G[2], G[2] + G[1], G[3] + G[3]};  // ∇u + ∇u'
          const double tau = q.cs * p->nu;   // lattice_viscosity(problem) = problem.ν
          const double cs = q.cs;
          const double factor = p->dom0 * p->dom1;
          for (int i = 0; i < Q; ++i) {
            const int xi[2] = {q.cx[i], q.cy[i]};
            double H[4];
            hermite_q(2, xi, csinv, H);
            fl[i] += -factor * q.w[i] * 0.5 * ((tau + 0.5) * cs) * dot_arr(H, S, 4);
          }
        } else if (strategy == 2) {  // TGV specialisation, analytical_offequilibrium.jl:50-87
          const Mat2 g = velocity_gradient(*p, X, Y, 0.0);
          const double S[4] = {g.m[0] + g.m[0], g.m[1] + g.m[2], g.m[2] + g.m[1], g.m[3] + g.m[3]};
          const double cs = q.cs;
          const double tau = cs * p->nu;
          const double tau_eff = tau + 0.5;
          for (int i = 0; i < Q; ++i) {
            const int xi[2] = {q.cx[i], q.cy[i]};
            double H[4];
            hermite_q(2, xi, csinv, H);
            const double fneq = q.w[i] * (((cs * tau_eff) * rho) * 1.0) / 2 * dot_arr(H, S, 4);
            fl[i] -= fneq;
          }
        }
      } else if (strategy == 3) {  // constant_density.jl
        const Vec2 v = lattice_velocity(*p, X, Y);
        const double u[2] = {v.x, v.y};
        hermite_equilibrium(q, 1.0, u, 1.0, fl);
      } else if (strategy == 4) {  // analytical_velocity_stress.jl
        const Vec2 v = lattice_velocity(*p, X, Y);
        const double u[2] = {v.x, v.y};
        hermite_equilibrium(q, 1.0, u, 1.0, fl);
        const Mat2 g = velocity_gradient(*p, X, Y, 0.0);
        const double s2 = p->u_max * p->u_max;
        double G[4];
        for (int k = 0; k < 4; ++k) G[k] = s2 * g.m[k];
        const double S[4] = {G[0] + G[0], G[1] + G[2], G[2] + G[1], G[3] + G[3]};
        const double cs = q.cs;
        const double tau = cs * p->nu;
        const double tau_eff = tau + 0.5;
        for (int i = 0; i < Q; ++i) {
          const int xi[2] = {q.cx[i], q.cy[i]};
          double H[4];
          hermite_q(2, xi, csinv, H);
          const double fneq = q.w[i] * (((cs * tau_eff) * 1.0) * 1.0) / 2 * dot_arr(H, S, 4);
          fl[i] += -fneq;
        }
      } else {
        return -1;
      }
      for (int i = 0; i < Q; ++i) f[x + (size_t)nx * (y + (size_t)ny * i)] = fl[i];
    }
  return 0;
}

// One collide! call on a lattice (no stream, no BC).
int orc_collide(int qid, const orc_problem* p, const orc_collision* cm, int nx, int ny,
                const double* fin, double* fout, double time) {
  Model m;
  m.q = make_quad(qid);
  m.prob = *p;
  m.cm = *cm;
  m.nx = nx;
  m.ny = ny;
  if (cm->force_kind) {
    orc_problem pp = *p;
    pp.nx = nx;
    pp.ny = ny;
    ranges(pp, m.xr, m.yr, &m.xstep, &m.ystep);
  }
  const size_t n = (size_t)nx * ny * m.q.Q;
  std::vector<double> a(fin, fin + n), b(n);
  collide(m, a, b, time);
  std::memcpy(fout, b.data(), n * sizeof(double));
  return 0;
}

int orc_stream(int qid, int nx, int ny, const double* f, double* fnew) {
  Model m;
  m.q = make_quad(qid);
  m.nx = nx;
  m.ny = ny;
  const size_t n = (size_t)nx * ny * m.q.Q;
  std::vector<double> a(f, f + n), b(n);
  stream(m, a, b);
  std::memcpy(fnew, b.data(), n * sizeof(double));
  return 0;
}

int orc_apply_bcs(int qid, int nx, int ny, int nbc, const orc_bc* bcs, double* fnew, const double* fold) {
  Model m;
  m.q = make_quad(qid);
  m.nx = nx;
  m.ny = ny;
  m.bcs.assign(bcs, bcs + nbc);
  const size_t n = (size_t)nx * ny * m.q.Q;
  std::vector<double> a(fnew, fnew + n), b(fold, fold + n);
  apply_bcs(m, a, b);
  std::memcpy(fnew, a.data(), n * sizeof(double));
  return 0;
}

// Processing reductions, TrackHydrodynamicErrors.next! (track_hydrodynamic_errors.jl:52-221):
// out = [error_ρ, error_u, error_p, error_σ_xx, error_σ_xy, error_σ_yy, error_σ_yx, mass,
// momentum, energy] for the lattice f at integer step t.
static void track_errors(const Model& m, const std::vector<double>& f, long t, double* out) {
  const Quad& q = m.q;
  const orc_problem& p = m.prob;
  const int nx = m.nx, ny = m.ny;
  const double time = t * delta_t(p);
  double D = m.ystep * m.xstep;
  if (nx == 1) {
    D = m.ystep;
    if (ny == 1) D = 1.0;
  } else if (ny == 1) {
    D = m.xstep;
  }
  const double D_ = D;
  double e_rho = 0, e_u = 0, e_p = 0, e_sxx = 0, e_sxy = 0, e_syy = 0, e_syx = 0;
  double tu2 = 0, tsxx = 0, tsyy = 0, tsxy = 0, tsyx = 0, tp2 = 0, mass = 0, mom = 0, en = 0;
  const double tau_p = q.cs * p.nu;  // τ = (1/c_s²)·ν (no + ½), track_hydrodynamic_errors.jl:148,176
  for (int x = 0; x < nx; ++x)
    for (int y = 0; y < ny; ++y) {
      const double X = m.xr[x], Y = m.yr[y];
      const double erho = density_a(p, q.cs, X, Y, time);
      const Vec2 eu = velocity_a(p, X, Y, time);
      const double ep = pressure_a(p, q.cs, X, Y, time);
      const Mat2 es = deviatoric_a(p, X, Y, time);
      tu2 += eu.x * eu.x + eu.y * eu.y;
      tsxx += es.m[0] * es.m[0];
      tsyy += es.m[3] * es.m[3];
      tsxy += es.m[2] * es.m[2];
      tsyx += es.m[1] * es.m[1];
      tp2 += ep * ep;
      double fl[37] = {0};
      for (int i = 0; i < q.Q; ++i) fl[i] = f[m.idx(x, y, i)];
      const double rho = density(q, fl);
      double u[2];
      velocity(q, fl, rho, u);
      double a2[4], aeq[4];
      second_moment(q, fl, a2);
      eq_coeff(2, q.cs, rho, u, 1.0, aeq);
      const double h = 1.0 / (2 * tau_p);
      double A2[4];
      for (int k = 0; k < 4; ++k) A2[k] = (a2[k] + h * aeq[k]) / (1 + 1 / (2 * tau_p));
      // P = a_2 - ρ (u u' - I)
      const double P00 = A2[0] - rho * (u[0] * u[0] - 1.0);
      const double P11 = A2[3] - rho * (u[1] * u[1] - 1.0);
      double s[4];
      deviatoric_tensor(q, tau_p, fl, rho, u, s);
      const double pr = (P00 + P11) / 2;
      const double ud[2] = {u[0] / p.u_max, u[1] / p.u_max};
      const double fac = 1 / (p.u_max * p.u_max);
      for (int k = 0; k < 4; ++k) s[k] = s[k] * fac;
      e_p += 1.0 * ((pr - ep) * (pr - ep));
      e_rho += 1.0 * ((rho - erho) * (rho - erho));
      e_u += 1.0 * ((ud[0] - eu.x) * (ud[0] - eu.x) + (ud[1] - eu.y) * (ud[1] - eu.y));
      e_sxx += 1.0 * ((es.m[0] - s[0]) * (es.m[0] - s[0]));
      e_sxy += 1.0 * ((es.m[2] - s[2]) * (es.m[2] - s[2]));
      e_syx += 1.0 * ((es.m[1] - s[1]) * (es.m[1] - s[1]));
      e_syy += 1.0 * ((es.m[3] - s[3]) * (es.m[3] - s[3]));
      mass += rho;
      mom += rho * (ud[0] + ud[1]);
      en += rho * (ud[0] * ud[0] + ud[1] * ud[1]);
    }
  out[0] = std::sqrt(e_rho);
  out[1] = std::sqrt(e_u / tu2);
  out[2] = std::sqrt(e_p / tp2);
  out[3] = std::sqrt(e_sxx / tsxx);
  out[4] = std::sqrt(e_sxy / tsxy);
  out[5] = std::sqrt(e_syy / tsyy);
  out[6] = std::sqrt(e_syx / tsyx);
  out[7] = D_ * mass;
  out[8] = D_ * mom;
  out[9] = D_ * en;
}

int orc_track_errors(int qid, const orc_problem* p, const double* f, long t, double* out) {
  Model m;
  m.q = make_quad(qid);
  m.prob = *p;
  m.nx = p->nx;
  m.ny = p->ny;
  ranges(*p, m.xr, m.yr, &m.xstep, &m.ystep);
  std::vector<double> fv(f, f + (size_t)m.nx * m.ny * m.q.Q);
  track_errors(m, fv, t, out);
  return 0;
}

// CompareWithAnalyticalSolution process! (processing_methods.jl:142-269):
// out = [density, momentum, total_energy, kinetic_energy, internal_energy, density_a,
//        momentum_a, total_energy_a, kinetic_energy_a, internal_energy_a, error_u, error_p]
static void compare_process(const Model& m, const std::vector<double>& f, double time, double* out) {
  const Quad& q = m.q;
  const orc_problem& p = m.prob;
  double td = 0, tm = 0, te = 0, tke = 0, tie = 0, etd = 0, etm = 0, ete = 0, etke = 0, etie = 0;
  double eu = 0, ep = 0;
  for (int x = 0; x < m.nx; ++x)
    for (int y = 0; y < m.ny; ++y) {
      double fl[37] = {0};
      for (int i = 0; i < q.Q; ++i) fl[i] = f[m.idx(x, y, i)];
      const double rho = density(q, fl);
      double u[2];
      velocity(q, fl, rho, u);
      const double T = pressure(q, fl, rho, u) / rho;
      const double pr = pressure(q, fl, rho, u);
      const double ud[2] = {u[0] / p.u_max, u[1] / p.u_max};
      td += 1.0 * rho;
      tm += 1.0 * (ud[0] + ud[1]) * rho;
      const double ke = 1.0 * (ud[0] * ud[0] + ud[1] * ud[1]) * rho;
      tke += 1.0 * ke;
      tie += 1.0 * T;
      te += 1.0 * (ke + T);
      const double X = m.xr[x], Y = m.yr[y];
      const double erho = density_a(p, q.cs, X, Y, time);
      const double epr = pressure_a(p, q.cs, X, Y, time);
      const Vec2 ev = velocity_a(p, X, Y, time);
      const double eT = epr / erho;
      const double eke = ev.x * ev.x + ev.y * ev.y;
      etd += erho;
      etm += erho * (ev.x + ev.y);
      etke += eke;
      etie += eT;
      ete += eke + eT;
      const double opp = m.ystep * m.xstep;
      eu += opp * ((ud[0] - ev.x) * (ud[0] - ev.x) + (ud[1] - ev.y) * (ud[1] - ev.y));
      ep += opp * ((pr - epr) * (pr - epr));
    }
  out[0] = td; out[1] = tm; out[2] = te; out[3] = tke; out[4] = tie;
  out[5] = etd; out[6] = etm; out[7] = ete; out[8] = etke; out[9] = etie;
  out[10] = std::sqrt(eu); out[11] = std::sqrt(ep);
}

// ---------------------------------------------------------------------------------------
// simulate(model, time): lattice_boltzmann_model.jl:60-77 with the processing method
// next!(pm, q, f, t) of the reference:
//   pm_kind 0: TrackHydrodynamicErrors (track_hydrodynamic_errors.jl:52-242)
//   pm_kind 1: CompareWithAnalyticalSolution (processing_methods.jl:92-140)
//   pm_kind 2: ProcessIterativeInitialization (process_iterative_initialization.jl)
//   pm_kind 3: none (never stops, records nothing)
// stop kinds: 0 none, 1 MeanVelocity(tol), 2 VelocityConvergence(tol), 3 DensityConvergence(ϵ)
// ---------------------------------------------------------------------------------------
typedef struct {
  int pm_kind;
  int should_process;
  long n_steps;
  int stop_kind;
  double stop_tol;
  int has_problem;   // false ⇒ Δt = 0 (pm without a :problem field)
  int nthreads;
} orc_processing;

typedef struct {
  long timestep;
  double v[16];
} orc_row;

int orc_simulate(int qid, const orc_problem* p, const orc_collision* cm, int nbc, const orc_bc* bcs,
                 const orc_processing* pm, long t_first, long t_last, double* f_inout,
                 orc_row* rows, int max_rows, int* n_rows, long* stopped_at) {
  Model m;
  m.q = make_quad(qid);
  m.prob = *p;
  m.cm = *cm;
  m.bcs.assign(bcs, bcs + nbc);
  m.nx = p->nx;
  m.ny = p->ny;
  m.nthreads = pm->nthreads > 0 ? pm->nthreads : 1;
  ranges(*p, m.xr, m.yr, &m.xstep, &m.ystep);
  const int Q = m.q.Q;
  const size_t n = (size_t)m.nx * m.ny * Q;
  m.f_stream.assign(f_inout, f_inout + n);
  m.f_collision = m.f_stream;
  if (cm->kind == 3) {  // IterativeInitializationCollisionModel(q, τ, problem)
    m.nonlinear.assign(n, 0.0);
    for (int x = 0; x < m.nx; ++x)
      for (int y = 0; y < m.ny; ++y) {
        const Vec2 v = lattice_velocity(*p, m.xr[x], m.yr[y]);
        const double u2 = v.x * v.x + v.y * v.y;
        for (int i = 0; i < Q; ++i) {
          const double cu = m.q.cx[i] * v.x + m.q.cy[i] * v.y;
          const double cs = m.q.cs;
          const double a1 = cs * cu;
          const double a2 = (cs * cs) * (cu * cu) - cs * u2;
          m.nonlinear[m.idx(x, y, i)] = m.q.w[i] * 1.0 * (a1 + a2 / 2);
        }
      }
  }
  const double dt = pm->has_problem ? delta_t(*p) : 0.0;
  // stop criterion state
  double old_mean = 0.0;
  std::vector<double> old_u;
  if (pm->stop_kind == 2) old_u.assign((size_t)m.nx * m.ny * 2, 0.0);
  std::vector<double> rho_old((size_t)m.nx * m.ny, 0.0), rho_new((size_t)m.nx * m.ny, 0.0);
  *n_rows = 0;
  *stopped_at = -1;

  auto should_stop = [&](const std::vector<double>& f) -> bool {
    const Quad& q = m.q;
    if (pm->stop_kind == 1) {  // MeanVelocityStoppingCriteria, stopping_criteria.jl:17-56
      double um = 0.0;
      long cnt = 0;
      for (int x = 0; x < m.nx; ++x)
        for (int y = 0; y < m.ny; ++y) {
          cnt += 1;
          double fl[37] = {0};
          for (int i = 0; i < Q; ++i) fl[i] = f[m.idx(x, y, i)];
          const double rho = density(q, fl);
          double u[2];
          velocity(q, fl, rho, u);
          um += u[0];
        }
      um /= cnt;
      const double conv = std::fabs(um / old_mean - 1);
      if (conv < pm->stop_tol) return true;
      if (std::isnan(um)) return true;
      old_mean = um;
      return false;
    } else if (pm->stop_kind == 2) {  // VelocityConvergenceStoppingCriteria, :72-115
      double err = 0.0, oldn = 0.0;
      for (int x = 0; x < m.nx; ++x)
        for (int y = 0; y < m.ny; ++y) {
          double fl[37] = {0};
          for (int i = 0; i < Q; ++i) fl[i] = f[m.idx(x, y, i)];
          const double rho = density(q, fl);
          double u[2];
          velocity(q, fl, rho, u);
          double* uo = &old_u[2 * ((size_t)x + (size_t)m.nx * y)];
          err += ((u[0] - uo[0]) * (u[0] - uo[0]) + (u[1] - uo[1]) * (u[1] - uo[1]));
          oldn += uo[0] * uo[0] + uo[1] * uo[1];
          uo[0] = u[0];
          uo[1] = u[1];
        }
      const double conv = std::sqrt(err) / oldn;
      if (conv < pm->stop_tol) return true;
      if (std::isnan(conv)) return true;
      return false;
    } else if (pm->stop_kind == 3) {  // DensityConvergence, density_convergence.jl:6-17
      const int x = m.nx - 1, y = m.ny - 1;  // `for x_idx in nx, y_idx in ny`: one node only
      const size_t k = x + (size_t)m.nx * y;
      rho_old[k] = rho_new[k];
      double fl[37] = {0};
      for (int i = 0; i < Q; ++i) fl[i] = f[m.idx(x, y, i)];
      rho_new[k] = density(q, fl);
      double s = 0.0;
      for (size_t j = 0; j < rho_new.size(); ++j) s += (rho_new[j] - rho_old[j]) * (rho_new[j] - rho_old[j]);
      const double drho = std::sqrt(s);
      return drho < pm->stop_tol || drho > 100.0;
    }
    return false;
  };

  auto push_row = [&](long ts, const double* v, int nv) {
    if (*n_rows < max_rows) {
      rows[*n_rows].timestep = ts;
      for (int k = 0; k < nv; ++k) rows[*n_rows].v[k] = v[k];
      for (int k = nv; k < 16; ++k) rows[*n_rows].v[k] = 0.0;
    }
    *n_rows += 1;
  };

  auto next = [&](long t) -> bool {
    const std::vector<double>& f = m.f_stream;
    if (pm->pm_kind == 0) {  // TrackHydrodynamicErrors
      bool stop = false;
      if (t % 100 == 0 && should_stop(f)) stop = true;
      if (!stop && t != pm->n_steps && !pm->should_process) return false;
      double out[10];
      track_errors(m, f, t, out);
      push_row(t, out, 10);
      return stop;
    } else if (pm->pm_kind == 1) {  // CompareWithAnalyticalSolution
      if (t % 100 == 0 && should_stop(f)) {
        double out[12];
        compare_process(m, f, t * delta_t(*p), out);
        push_row(t, out, 12);
        return true;
      }
      if (!pm->should_process && t != pm->n_steps) return false;
      double out[12];
      compare_process(m, f, t * delta_t(*p), out);
      push_row(t, out, 12);
      return false;
    } else if (pm->pm_kind == 2) {  // ProcessIterativeInitialization
      return should_stop(f);
    }
    return false;
  };

  for (long t = t_first; t <= t_last; ++t) {
    collide(m, m.f_stream, m.f_collision, t * dt);
    stream(m, m.f_collision, m.f_stream);
    apply_bcs(m, m.f_stream, m.f_collision);
    if (next(t + 1)) {
      *stopped_at = t + 1;
      std::memcpy(f_inout, m.f_stream.data(), n * sizeof(double));
      return 0;
    }
  }
  next(t_last + 1);
  std::memcpy(f_inout, m.f_stream.data(), n * sizeof(double));
  return 0;
}

// Bare time loop (collide → stream → BCs), no processing: the CPU baseline workload.
int orc_run(int qid, const orc_problem* p, const orc_collision* cm, int nbc, const orc_bc* bcs,
            long t_first, long t_last, double dt, int nthreads, double* f_inout) {
  Model m;
  m.q = make_quad(qid);
  m.prob = *p;
  m.cm = *cm;
  m.bcs.assign(bcs, bcs + nbc);
  m.nx = p->nx;
  m.ny = p->ny;
  m.nthreads = nthreads > 0 ? nthreads : 1;
  ranges(*p, m.xr, m.yr, &m.xstep, &m.ystep);
  const size_t n = (size_t)m.nx * m.ny * m.q.Q;
  m.f_stream.assign(f_inout, f_inout + n);
  m.f_collision = m.f_stream;
  for (long t = t_first; t <= t_last; ++t) {
    collide(m, m.f_stream, m.f_collision, t * dt);
    stream(m, m.f_collision, m.f_stream);
    apply_bcs(m, m.f_stream, m.f_collision);
  }
  std::memcpy(f_inout, m.f_stream.data(), n * sizeof(double));
  return 0;
}

// Forward-mode derivative of a field loss through the time loop, for the gradient checks of
// the adjoint: f_0 = equilibrium(1, u0) per node (maxwell_boltzmann_equilibrium.jl:12-66),
// then `nsteps` times collide! (SRT kind 0 / TRT kind 1 / MRT kind 2 of a second-order set, with
// the uniform lattice force F, as srt.jl:18-62 / trt.jl:42-97 / mrt.jl:56-118; MRT: tau = (τs[1],
// τs[2])) and the periodic stream! (stream.jl:18-30), and
//     L = Σ_nodes (u_x - ut_x)² + (u_y - ut_y)²,   u = velocity!(f_T) (moments.jl:1-19).
// Every value is a Dual whose derivative part is seeded with the direction
// (dτ_0, dτ_1, dF_x, dF_y) = seed and du0 for u0 (null: zero), so out = (L, dL/dε along it).
// u0, ut, du0: arrays [2][ny][nx] (component, y, x).
int orc_tangent_loss(int qid, int kind, const double* tau, const double* F, int nx, int ny, const double* u0,
                     const double* ut, const double* seed, const double* du0, long nsteps, int nthreads,
                     const orc_bc* bcs, int nbc, double* out) {
  if (kind < 0 || kind > 2 || nx <= 0 || ny <= 0 || nsteps < 0 || nbc < 0 || (nbc > 0 && !bcs)) return -1;
  const std::vector<orc_bc> bclist(bcs, bcs + nbc);
  const Quad q = make_quad(qid);
  if (kind == 2 && q.order / 2 != 2) return -1;
  double Hs[5][37][16];
  if (kind == 2)
    for (int nh = 1; nh <= 2; ++nh)
      for (int i = 0; i < q.Q; ++i) {
        const int xi[2] = {q.cx[i], q.cy[i]};
        hermite_q(nh, xi, 1.0 / q.cs, Hs[nh][i]);
      }
  const int Q = q.Q;
  const size_t nn = (size_t)nx * ny, n = nn * Q;
  auto idx = [&](int x, int y, int i) { return (size_t)x + (size_t)nx * ((size_t)y + (size_t)ny * i); };
  const Dual t0(tau[0], seed[0]), t1(tau[1], seed[1]), Fx(F[0], seed[2]), Fy(F[1], seed[3]);
  const bool force = F[0] != 0.0 || F[1] != 0.0 || seed[2] != 0.0 || seed[3] != 0.0;
  std::vector<Dual> a(n), b(n);
  for (int y = 0; y < ny; ++y)
    for (int x = 0; x < nx; ++x) {
      const size_t k = (size_t)y * nx + x;
      const Dual u[2] = {Dual(u0[k], du0 ? du0[k] : 0.0), Dual(u0[nn + k], du0 ? du0[nn + k] : 0.0)};
      Dual feq[37];
      equilibrium(q, Dual(1.0), u, feq);
      for (int i = 0; i < Q; ++i) a[idx(x, y, i)] = feq[i];
    }
  for (long t = 0; t < nsteps; ++t) {
#pragma omp parallel for schedule(static) num_threads(nthreads) if (nthreads > 1)
    for (int x = 0; x < nx; ++x) {
      Dual f[37], o[37];
      for (int y = 0; y < ny; ++y) {
        for (int i = 0; i < Q; ++i) f[i] = a[idx(x, y, i)];
        if (kind == 2) collide_mrt2_node<Dual>(q, Hs, t0, t1, force, Fx, Fy, f, o);
        else collide_srt_trt_node<Dual>(q, kind, t0, t1, force, Fx, Fy, f, o);
        for (int i = 0; i < Q; ++i) b[idx(x, y, i)] = o[i];
      }
    }
    stream_periodic(q, nx, ny, b.data(), a.data(), nthreads);
    apply_bcs_t<Dual>(q, nx, ny, bclist, a.data(), b.data());
  }
  Dual L = 0.0;
  for (int y = 0; y < ny; ++y)
    for (int x = 0; x < nx; ++x) {
      const size_t k = (size_t)y * nx + x;
      Dual f[37], u[2];
      for (int i = 0; i < Q; ++i) f[i] = a[idx(x, y, i)];
      velocity(q, (const Dual*)f, density(q, (const Dual*)f), u);
      const Dual ex = u[0] - ut[k], ey = u[1] - ut[nn + k];
      L += ex * ex + ey * ey;
    }
  out[0] = L.v;
  out[1] = L.d;
  return 0;
}

int orc_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // extern "C"
