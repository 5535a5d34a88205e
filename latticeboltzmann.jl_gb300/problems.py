"""Fluid-flow problems of LatticeBoltzmann.jl (L3): analytic fields, forces, unit conversion
and boundary-condition lists, vectorised over numpy coordinate arrays.

  FluidFlowProblem defaults        src/problems/problems.jl
  TaylorGreenVortex                src/problems/taylor_green_vortex.jl
  TGV                              src/problems/second_order_convergence.jl
  PoiseuilleFlow                   src/problems/poiseuille.jl
  CouetteFlow                      src/problems/couette_flow.jl
  DecayingShearFlow                src/problems/decaying_shear_flow.jl
  LidDrivenCavityFlow              src/problems/lid_driven_cavity.jl
  LinearizedThermalDiffusion,
  LinearizedTransverseShearWave    src/problems/linear_hydrodynamics_modes.jl

Constructors keep the reference's keyword defaults and its size overrides (PoiseuilleFlow
forces NX = 3, CouetteFlow NX = 1, DecayingShearFlow NY = 3 when k_y = 0).  Each class
also accepts the positional field list of the reference struct through ``.fields(...)``.
User problem types subclass FluidFlowProblem and override the analytic methods, as the
reference's tests do (test/initial_conditions.jl:12-87).
"""
from __future__ import annotations

import functools
import math

import numpy as np

from .boundary_conditions import BounceBack, MovingWall, North, South, East, West


class FluidFlowProblem:
    NX: int
    NY: int
    u_max: float
    ν: float
    domain_size: tuple
    static = False

    # ---- unit conversion (problems.jl:79-119) ---------------------------------------------
    def delta_x(self):
        if self.NX > self.NY:
            return self.domain_size[0] * (1 / self.NX)
        return self.domain_size[1] * (1 / self.NY)

    def delta_t(self):
        return self.delta_x() * self.u_max

    def viscosity(self):
        dx = self.delta_x()
        return self.ν * (dx * dx) / self.delta_t()

    def lattice_viscosity(self):
        return self.ν

    def has_external_force(self):
        return False

    def boundary_conditions(self):
        return []

    # ---- analytic fields (defaults of problems.jl) ----------------------------------------
    def density(self, q, x, y, t=0.0):
        return np.ones(np.broadcast(x, y).shape)

    def pressure(self, q, x, y, t=0.0):
        return np.ones(np.broadcast(x, y).shape)

    def velocity(self, x, y, t=0.0):
        z = np.zeros(np.broadcast(x, y).shape)
        return z, z.copy()

    def velocity_gradient(self, x, y, t=0.0):
        """[[u_x, v_x], [u_y, v_y]] as an array of shape (2, 2) + shape(x)."""
        return np.zeros((2, 2) + np.broadcast(x, y).shape)

    def force(self, x, y, t=0.0):
        z = np.zeros(np.broadcast(x, y).shape)
        return z, z.copy()

    def deviatoric_tensor(self, q, x, y, t=0.0):
        """σ = -ν [2 a11, a12 + a21; a12 + a21, 2 a22] (problems.jl:30-46)."""
        a = self.velocity_gradient(x, y, t)
        nu = self.viscosity()
        s = np.empty_like(a)
        s[0, 0] = -nu * (2 * a[0, 0])
        s[0, 1] = -nu * (a[0, 1] + a[1, 0])
        s[1, 0] = -nu * (a[0, 1] + a[1, 0])
        s[1, 1] = -nu * (2 * a[1, 1])
        return s

    def __repr__(self):
        return f"{type(self).__name__}(NX={self.NX}, NY={self.NY})"


# ---------------------------------------------------------------------------------------
# reference free functions
# ---------------------------------------------------------------------------------------
def _linspace(a: float, b: float, n: int):
    """Julia range(a, stop=b, length=n) for Float64: values computed in extended precision
    and rounded (Julia uses TwicePrecision arithmetic); a length-1 range has step 0."""
    if n == 1:
        return np.array([a]), 0.0
    la, lb = np.longdouble(a), np.longdouble(b)
    st = (lb - la) / np.longdouble(n - 1)
    vals = (la + st * np.arange(n, dtype=np.longdouble)).astype(np.float64)
    return vals, float(st)


def _ranges(NX, NY, d0, d1):
    """Node coordinates of a lattice; small lattices (the points of a sweep share them) are cached."""
    if NX * NY <= 1 << 16:
        return _ranges_cached(NX, NY, d0, d1)
    return _ranges_build(NX, NY, d0, d1)


@functools.lru_cache(maxsize=512)
def _ranges_cached(NX, NY, d0, d1):
    return _ranges_build(NX, NY, d0, d1)


def _ranges_build(NX, NY, d0, d1):
    dx = d0 / NX
    dy = d1 / NY
    xr, xs = _linspace(dx / 2, d0 - dx / 2, NX)
    yr, ys = _linspace(dy / 2, d0 - dy / 2, NY)
    X, Y = np.meshgrid(xr, yr)
    for a in (xr, yr, X, Y):
        a.setflags(write=False)  # shared between problems of one shape
    return xr, yr, xs, ys, X, Y


def problem_range(problem):
    """The reference's range(problem) (problems.jl:18-26): cell-centred node coordinates.
    Like the reference, the y range ends at domain_size[1] - Δy/2 using the FIRST domain
    extent.  Returns (x_range, y_range, x_step, y_step)."""
    xr, yr, xs, ys, _, _ = _ranges(int(problem.NX), int(problem.NY), float(problem.domain_size[0]),
                                   float(problem.domain_size[1]))
    return xr, yr, xs, ys


def delta_t(problem):
    return problem.delta_t()


def delta_x(problem):
    return problem.delta_x()


def viscosity(problem):
    return problem.viscosity()


def lattice_viscosity(problem):
    return problem.lattice_viscosity()


def has_external_force(problem):
    return problem.has_external_force()


def boundary_conditions(problem):
    return problem.boundary_conditions()


def lattice_velocity(q, problem, x, y, t=0.0):
    ux, uy = problem.velocity(x, y, t)
    return problem.u_max * ux, problem.u_max * uy


def lattice_density(q, problem, x, y, t=0.0):
    return problem.density(q, x, y, t)


def lattice_pressure(q, problem, x, y, t=0.0):
    return problem.u_max ** 2 * problem.pressure(q, x, y, t)


def lattice_temperature(q, problem, x, y, t=0.0):
    # problems.jl:105-106: pressure / density at t = 0
    return problem.pressure(q, x, y) / problem.density(q, x, y)


def node_grid(problem):
    """Coordinate arrays X, Y of shape (NY, NX) (row y, column x)."""
    return _ranges(int(problem.NX), int(problem.NY), float(problem.domain_size[0]),
                   float(problem.domain_size[1]))[4:]


def lattice_force_field(problem, t=0.0, nodes=None):
    """lattice_force(problem, x_idx, y_idx, t) at every node, shape (2, NY, NX)
    (problems.jl:62-74, 103-104); with `nodes` = 1, at node (1, 1) only, shape (2, 1, 1)."""
    X, Y = node_grid(problem)
    if nodes == 1:
        X, Y = X[:1, :1], Y[:1, :1]
    Fx, Fy = problem.force(X, Y, t)
    s = problem.u_max * problem.delta_t()
    out = np.empty((2,) + X.shape)
    out[0] = s * np.broadcast_to(Fx, X.shape)
    out[1] = s * np.broadcast_to(Fy, X.shape)
    return out


def analytic_fields(q, problem, t):
    """Expected ρ, u, p, σ of the problem at physical time t on its lattice, as a dict of
    (NY, NX) arrays; the inputs of the error-norm reductions."""
    X, Y = node_grid(problem)
    rho = np.broadcast_to(problem.density(q, X, Y, t), X.shape).astype(np.float64)
    ux, uy = problem.velocity(X, Y, t)
    p = np.broadcast_to(problem.pressure(q, X, Y, t), X.shape).astype(np.float64)
    s = problem.deviatoric_tensor(q, X, Y, t)
    out = np.empty((8,) + X.shape)  # one block, so the eight planes travel in one copy
    for k, a in enumerate((rho, ux, uy, p, s[0, 0], s[1, 0], s[0, 1], s[1, 1])):
        out[k] = a
    return dict(zip(("rho", "ux", "uy", "p", "sxx", "syx", "sxy", "syy"), out))


# ---------------------------------------------------------------------------------------
# problems
# ---------------------------------------------------------------------------------------
class TaylorGreenVortex(FluidFlowProblem):
    """TaylorGreenVortex(ν=1/6, scale=2, NX=16 scale, NY=NX, domain=(2π, 2π); static=True,
    A=1, B=-1, a=1, b=1) with u_max = 0.01 / scale (taylor_green_vortex.jl:14-34)."""

    def __init__(self, ν=1.0 / 6.0, scale=2, NX=None, NY=None, domain_size=(2 * math.pi, 2 * math.pi), *,
                 static=True, A=1.0, B=-1.0, a=1.0, b=1.0):
        self.NX = 16 * scale if NX is None else NX
        self.NY = self.NX if NY is None else NY
        self.rho_0 = 1.0
        self.u_max = 0.01 / scale
        self.ν = ν
        self.domain_size = tuple(float(d) for d in domain_size)
        self.static = bool(static)
        self.A, self.B, self.a, self.b = float(A), float(B), float(a), float(b)

    def decay(self, x, y, t):
        if self.static:
            return 1.0
        return math.exp(-(self.a ** 2 + self.b ** 2) * self.viscosity() * t)

    def pressure(self, q, x, y, t=0.0):
        d = self.decay(x, y, t)
        P = -(1 / 4) * self.rho_0 * (d * d) * ((self.A * self.A) * np.cos(2 * self.a * x)
                                                + (self.B * self.B) * np.cos(2 * self.b * y))
        return 1.0 + q.speed_of_sound_squared * (self.u_max * self.u_max) * P

    def density(self, q, x, y, t=0.0):
        return self.pressure(q, x, y, t)

    def velocity(self, x, y, t=0.0):
        d = self.decay(x, y, t)
        return (d * (self.A * np.cos(self.a * x) * np.sin(self.b * y)),
                d * (self.B * np.sin(self.a * x) * np.cos(self.b * y)))

    def velocity_gradient(self, x, y, t=0.0):
        a, A, b, B = self.a, self.A, self.b, self.B
        s = self.decay(x, y, t)
        ux = -a * A * np.sin(a * x) * np.sin(b * y)
        vy = -b * B * np.sin(a * x) * np.sin(b * y)
        uy = b * A * np.cos(a * x) * np.cos(b * y)
        vx = a * B * np.cos(a * x) * np.cos(b * y)
        return np.array([[s * ux, s * vx], [s * uy, s * vy]])

    def force(self, x, y, t=0.0):
        if self.static:
            vx, vy = self.velocity(x, y, 0.0)
            s = 2 * self.viscosity()
            return s * vx, s * vy
        return super().force(x, y, t)

    def has_external_force(self):
        return self.static


class TGV(FluidFlowProblem):
    """TGV(q, τ, scale=2, NX=16 scale, NY=NX, u_max=0.02/scale): the lattice-unit Taylor-Green
    vortex of the convergence studies (second_order_convergence.jl:1-26).  The u_max argument
    is stored as u_0; the struct's own u_max is 1, Δx = Δt = 1."""

    def __init__(self, q, τ, scale=2, NX=None, NY=None, u_max=None):
        self.q = q
        self.rho_0 = 1.0
        self.u_max = 1.0
        self.u_0 = 0.02 / scale if u_max is None else float(u_max)
        self.τ = float(τ)
        self.ν = (self.τ - 0.5) / q.speed_of_sound_squared
        self.NX = 16 * scale if NX is None else NX
        self.NY = self.NX if NY is None else NY
        self.static = False
        self.domain_size = (1.0, 1.0)

    def delta_x(self):
        return 1.0

    def delta_t(self):
        return 1.0

    def viscosity(self):
        return self.ν

    def _k(self):
        kx = 2 * math.pi / self.NX
        ky = 2 * math.pi / self.NY
        td = 1 / (self.ν * (kx * kx + ky * ky))
        return kx, ky, td

    def decay_time(self):
        return self._k()[2]

    def density(self, q, x, y, t=0.0):
        kx, ky, td = self._k()
        X, Y = x * self.NX, y * self.NY
        return self.rho_0 * (1.0 - q.speed_of_sound_squared * ((self.u_0 * self.u_0) / 4)
                             * ((ky / kx) * np.cos(2 * kx * X) + (kx / ky) * np.cos(2 * ky * Y))
                             * math.exp(-2 * t / td))

    def pressure(self, q, x, y, t=0.0):
        kx, ky, td = self._k()
        X, Y = x * self.NX, y * self.NY
        return self.rho_0 - q.speed_of_sound_squared * 1.0 * ((self.u_0 * self.u_0) / 4) * \
            ((ky / kx) * np.cos(2 * kx * X) + (kx / ky) * np.cos(2 * ky * Y)) * math.exp(-2 * t / td)

    def velocity(self, x, y, t=0.0):
        kx, ky, td = self._k()
        X, Y = x * self.NX, y * self.NY
        s = self.u_0 * math.exp(-t / td)
        return (s * (-math.sqrt(ky / kx) * np.cos(kx * X) * np.sin(ky * Y)),
                s * (math.sqrt(kx / ky) * np.sin(kx * X) * np.cos(ky * Y)))

    def velocity_gradient(self, x, y, t=0.0):
        kx, ky, td = self._k()
        X, Y = x * self.NX, y * self.NY
        ux = math.sqrt(ky * kx) * np.sin(kx * X) * np.sin(ky * Y)
        vy = -math.sqrt(ky * kx) * np.sin(kx * X) * np.sin(ky * Y)
        uy = -math.sqrt((ky * ky * ky) / kx) * np.cos(kx * X) * np.cos(ky * Y)
        vx = math.sqrt((kx * kx * kx) / ky) * np.cos(kx * X) * np.cos(ky * Y)
        s = math.exp(-t / td) * self.u_0
        return np.array([[s * ux, s * vx], [s * uy, s * vy]])


def decay_time(problem):
    """t_d = 1 / (ν (k_x² + k_y²)) (second_order_convergence.jl:123-128)."""
    nu = problem.viscosity()
    kx = 2 * math.pi / problem.NX
    ky = 2 * math.pi / problem.NY
    return 1 / (nu * (kx * kx + ky * ky))


class PoiseuilleFlow(FluidFlowProblem):
    """PoiseuilleFlow(ν=1/6, scale=2, NX=5 scale, NY=NX, domain=(1, 1)) with NX forced to 3 and
    u_max = 0.1 / scale (poiseuille.jl:12-26); body force ν_phys G along x; bounce-back walls
    North and South."""

    def __init__(self, ν=1.0 / 6.0, scale=2, NX=None, NY=None, domain_size=(1.0, 1.0), *, static=True):
        NX = 5 * scale if NX is None else NX
        self.NY = NX if NY is None else NY
        self.NX = 3
        self.rho_0 = 1.0
        self.u_max = 0.1 / scale
        self.ν = ν
        self.k = 1.0
        self.domain_size = tuple(float(d) for d in domain_size)
        self.G = 1.0

    @classmethod
    def fields(cls, rho_0, u_max, ν, NX, NY, k, domain_size, G):
        """The positional struct constructor PoiseuilleFlow(ρ0, u_max, ν, NX, NY, k, domain, G)."""
        p = cls.__new__(cls)
        p.rho_0, p.u_max, p.ν, p.NX, p.NY, p.k = float(rho_0), float(u_max), float(ν), int(NX), int(NY), float(k)
        p.domain_size = tuple(float(d) for d in domain_size)
        p.G = float(G)
        return p

    def delta_x(self):
        return self.domain_size[1] / self.NY

    def velocity(self, x, y, t=0.0):
        ux = y * (self.domain_size[1] - y) * (self.G / 2)
        return ux + 0.0 * x, np.zeros(np.broadcast(x, y).shape)

    def velocity_gradient(self, x, y, t=0.0):
        shp = np.broadcast(x, y).shape
        z = np.zeros(shp)
        uy = (self.domain_size[1] - 2 * y) * (self.G / 2) + 0.0 * x
        return np.array([[z, z], [uy, z]])

    def force(self, x, y, t=0.0):
        shp = np.broadcast(x, y).shape
        return np.full(shp, self.viscosity() * self.G), np.zeros(shp)

    def has_external_force(self):
        return True

    def boundary_conditions(self):
        return [BounceBack(North(), (1, self.NX), (1, self.NY)), BounceBack(South(), (1, self.NX), (1, self.NY))]


class CouetteFlow(FluidFlowProblem):
    """CouetteFlow(ν=1/6, scale=2, NX=5 scale, NY=NX, domain=(1, 1)) with NX forced to 1 and
    u_max = 0.01 / scale; bounce-back South, moving wall North (couette_flow.jl:10-25)."""

    def __init__(self, ν=1.0 / 6.0, scale=2, NX=None, NY=None, domain_size=(1.0, 1.0)):
        NX = 5 * scale if NX is None else NX
        self.NY = NX if NY is None else NY
        self.NX = 1
        self.rho_0 = 1.0
        self.u_max = 0.01 / scale
        self.ν = ν
        self.domain_size = tuple(float(d) for d in domain_size)

    def velocity(self, x, y, t=0.0):
        return y + 0.0 * x, np.zeros(np.broadcast(x, y).shape)

    def velocity_gradient(self, x, y, t=0.0):
        shp = np.broadcast(x, y).shape
        z = np.zeros(shp)
        return np.array([[z, z], [np.ones(shp), z]])

    def boundary_conditions(self):
        return [BounceBack(South(), (1, self.NX), (1, self.NY)),
                MovingWall(North(), (1, self.NX), (1, self.NY), [self.u_max, 0.0])]


class DecayingShearFlow(FluidFlowProblem):
    """DecayingShearFlow(ν=1/6, scale=2, NX=8 scale, NY=NX, domain=(2π, 2π); static=True, A=1,
    B=1, k_x=1, k_y=0) with u_max = 0.02 / scale; NY = 3 when k_y = 0, NX = 3 when k_x = 0
    (decaying_shear_flow.jl:14-36)."""

    def __init__(self, ν=1.0 / 6.0, scale=2, NX=None, NY=None, domain_size=(2 * math.pi, 2 * math.pi), *,
                 static=True, A=1.0, B=1.0, k_x=1.0, k_y=0.0):
        NX = 8 * scale if NX is None else NX
        NY = NX if NY is None else NY
        if k_y == 0.0:
            NY = 3
        if k_x == 0.0:
            NX = 3
        self.NX, self.NY = NX, NY
        self.rho_0 = 1.0
        self.u_max = 0.02 / scale
        self.ν = ν
        self.domain_size = tuple(float(d) for d in domain_size)
        self.static = bool(static)
        self.A, self.B, self.k_x, self.k_y = float(A), float(B), float(k_x), float(k_y)

    def decay(self, x, y, t):
        if self.static:
            return 1.0
        return math.exp(-1.0 * (self.k_x * self.k_x) * self.viscosity() * t)

    def pressure(self, q, x, y, t=0.0):
        s = np.sin(self.k_x * (x - self.A * t))
        d = self.decay(x, y, t)
        return 1 + self.B * 0.025 * q.speed_of_sound_squared * (self.u_max * self.u_max) * self.B * (s * s) * (d * d) \
            + 0.0 * y

    def velocity(self, x, y, t=0.0):
        A, B, kx, ky = self.A, self.B, self.k_x, self.k_y
        if self.static:
            return A * np.cos(ky * y - ky * B * t) + 0.0 * x, B * np.cos(kx * x - kx * A * t) + 0.0 * y
        nu = self.viscosity()
        return (A * np.cos(ky * y - ky * B * t) * math.exp(-1.0 * (ky * ky) * nu * t) + 0.0 * x,
                B * np.cos(kx * x - kx * A * t) * math.exp(-1.0 * (kx * kx) * nu * t) + 0.0 * y)

    def velocity_gradient(self, x, y, t=0.0):
        A, B, kx, ky = self.A, self.B, self.k_x, self.k_y
        shp = np.broadcast(x, y).shape
        z = np.zeros(shp)
        uy = -A * ky * np.sin(ky * (y - B * t)) + 0.0 * x
        vx = -B * kx * np.sin(kx * (x - A * t)) + 0.0 * y
        if not self.static:
            nu = self.viscosity()
            uy = uy * math.exp(-1.0 * (ky * ky) * nu * t)
            vx = vx * math.exp(-1.0 * (kx * kx) * nu * t)
        return np.array([[z, vx], [uy, z]])

    def force(self, x, y, t=0.0):
        if not self.static:
            return super().force(x, y, t)
        A, B, kx, ky = self.A, self.B, self.k_x, self.k_y
        nu = self.viscosity()
        return (nu * (ky * ky) * A * np.cos(ky * y - ky * B * t) + 0.0 * x,
                nu * (kx * kx) * B * np.cos(kx * x - kx * A * t) + 0.0 * y)

    def shear_force_params(self):
        """Coefficients of the time-dependent lattice force for the device
        (LBM_FORCE_SHEAR): Fx = c0 cos(c1 y - c2 t), Fy = c3 cos(c4 x - c5 t)."""
        s = self.u_max * self.delta_t()
        nu = self.viscosity()
        A, B, kx, ky = self.A, self.B, self.k_x, self.k_y
        return [s * (nu * (ky * ky) * A), ky, ky * B, s * (nu * (kx * kx) * B), kx, kx * A]

    def has_external_force(self):
        return self.static


class LidDrivenCavityFlow(FluidFlowProblem):
    """LidDrivenCavityFlow(ν=1/6, scale=2, NX=16 scale, NY=NX, domain=(1, 1)), u_max = 0.01 / scale;
    bounce-back East, South, West and a moving lid North (lid_driven_cavity.jl:10-66)."""

    def __init__(self, ν=1.0 / 6.0, scale=2, NX=None, NY=None, domain_size=(1.0, 1.0)):
        self.NX = 16 * scale if NX is None else NX
        self.NY = self.NX if NY is None else NY
        self.rho_0 = 1.0
        self.u_max = 0.01 / scale
        self.ν = ν
        self.domain_size = tuple(float(d) for d in domain_size)

    def boundary_conditions(self):
        r = ((1, self.NX), (1, self.NY))
        return [BounceBack(East(), *r), BounceBack(South(), *r), BounceBack(West(), *r),
                MovingWall(North(), *r, [self.u_max, 0.0])]


class LinearizedThermalDiffusion(FluidFlowProblem):
    """LinearizedThermalDiffusion(ν, κ, scale, NY=4 scale) (linear_hydrodynamics_modes.jl:23-121)."""

    def __init__(self, ν, κ, scale, NY=None):
        NY = 4 * scale if NY is None else NY
        self.ρ_0, self.θ_0, self.ρ̃, self.ũ = 1.0, 1.0, 0.001, 0.001
        self.ν, self.κ = float(ν), float(κ)
        self.domain_size = (2 * math.pi, 2 * math.pi)
        self.u_max = 0.01 / scale
        self.NX = self.NY = NY

    def delta_x(self):
        return self.domain_size[1] / self.NY

    def heat_diffusion(self):
        dx = self.delta_x()
        return self.κ * (dx * dx) / self.delta_t()

    def density(self, q, x, y, t=0.0):
        return self.ρ_0 + self.ρ̃ * np.sin(y) * math.exp(-self.heat_diffusion() * t) + 0.0 * x

    def pressure(self, q, x, y, t=0.0):
        return np.full(np.broadcast(x, y).shape, self.ρ_0 * self.θ_0)


class LinearizedTransverseShearWave(FluidFlowProblem):
    """LinearizedTransverseShearWave(ν, κ, scale, NY=8 scale) (linear_hydrodynamics_modes.jl:123-177)."""

    def __init__(self, ν, κ, scale, NY=None):
        NY = 8 * scale if NY is None else NY
        self.ρ_0, self.θ_0, self.ρ̃, self.ũ = 1.0, 1.0, 0.001, 0.001
        self.ν, self.κ = float(ν), float(κ)
        self.domain_size = (2 * math.pi, 2 * math.pi)
        self.u_max = 0.01 / scale
        self.NX = self.NY = NY

    def delta_x(self):
        return self.domain_size[1] / self.NY

    def density(self, q, x, y, t=0.0):
        return np.full(np.broadcast(x, y).shape, self.ρ_0)

    def pressure(self, q, x, y, t=0.0):
        return np.full(np.broadcast(x, y).shape, self.θ_0)

    def velocity(self, x, y, t=0.0):
        return self.ũ * np.sin(y) * math.exp(-self.viscosity() * t) + 0.0 * x, np.zeros(np.broadcast(x, y).shape)


class ShearWave(FluidFlowProblem):
    """Lattice-unit transverse shear wave u_x = u0 sin(2π y / NY) e^{-ν k² t}, u_y = 0, ρ = 1,
    on an NX x NY periodic lattice with Δx = Δt = 1 (so `viscosity` is the lattice ν).  A
    user problem type in the sense of the reference's FluidFlowProblem extension mechanism;
    it is the analytic reference of the D2Q37 regularised-MRT shear-wave runs."""

    def __init__(self, NX, NY, ν, u0=0.01):
        self.NX, self.NY = int(NX), int(NY)
        self.ν = float(ν)
        self.u_0 = float(u0)
        self.u_max = 1.0
        self.domain_size = (float(NX), float(NY))

    def delta_x(self):
        return 1.0

    def delta_t(self):
        return 1.0

    def viscosity(self):
        return self.ν

    def velocity(self, x, y, t=0.0):
        k = 2 * math.pi / self.NY
        return self.u_0 * np.sin(k * y) * math.exp(-self.ν * (k * k) * t) + 0.0 * x, np.zeros(np.broadcast(x, y).shape)

    def velocity_gradient(self, x, y, t=0.0):
        k = 2 * math.pi / self.NY
        shp = np.broadcast(x, y).shape
        z = np.zeros(shp)
        uy = self.u_0 * k * np.cos(k * y) * math.exp(-self.ν * (k * k) * t) + 0.0 * x
        return np.array([[z, z], [uy, z]])
