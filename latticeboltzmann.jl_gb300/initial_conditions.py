"""Initial conditions of LatticeBoltzmann.jl (src/initial_conditions.jl and
src/initial_conditions/*.jl), evaluated over the whole lattice with numpy.

  ZeroVelocityInitialCondition            initial_conditions.jl:38-53   f = w
  AnalyticalEquilibrium                   analytical_equilibrium.jl     f = f_eq(ρ, u, T) (default)
  AnalyticalEquilibriumAndOffEquilibrium  analytical_offequilibrium.jl  + stress term (generic and TGV forms)
  ConstantDensity                         constant_density.jl           f_eq(1, u, 1)
  AnalyticalVelocityAndStress             analytical_velocity_stress.jl f_eq(1, u, 1) + stress term
  IterativeInitializationMeiEtAl(τ, ϵ)    mei_et_al.jl                  iterative, run on the device

`initialize(strategy, q, problem)` returns the populations in the Julia layout as a numpy
array of shape (Q, NY, NX) (element [i, y, x] is f[x+1, y+1, i+1] of the reference).
"""
from __future__ import annotations

import numpy as np

from . import kinetics as K
from .problems import TGV, lattice_velocity, node_grid


class InitializationStrategy:
    pass


class ZeroVelocityInitialCondition(InitializationStrategy):
    pass


class AnalyticalEquilibrium(InitializationStrategy):
    pass


class AnalyticalEquilibriumAndOffEquilibrium(InitializationStrategy):
    pass


class ConstantDensity(InitializationStrategy):
    pass


class AnalyticalVelocityAndStress(InitializationStrategy):
    pass


class AnalyticalVelocity(InitializationStrategy):
    """Present in the reference's API but its initial_condition calls an undefined
    pressure(problem, x, y) method (analytical_velocity.jl:29); not usable there either."""


class IterativeInitializationMeiEtAl(InitializationStrategy):
    def __init__(self, τ=1.0, ϵ=1e-7):
        self.τ = float(τ)
        self.ϵ = float(ϵ)


def IterativeInitialization():
    return IterativeInitializationMeiEtAl(1.0, 1e-7)


def default_strategy(problem):
    """InitializationStrategy(problem) = AnalyticalEquilibrium() (initial_conditions.jl:5)."""
    return AnalyticalEquilibrium()


def _dot_sym(H, S):
    # dot(H, S) over a 2x2 matrix in column-major order: H11 S11 + H21 S21 + H12 S12 + H22 S22
    acc = 0.0 + H[0, 0] * S[0, 0]
    acc = acc + H[1, 0] * S[1, 0]
    acc = acc + H[0, 1] * S[0, 1]
    acc = acc + H[1, 1] * S[1, 1]
    return acc


def initial_fields(strategy, q, problem):
    """The macroscopic planes from which `initialize` builds f, for the device-side build
    (DeviceLattice.initialize_fields / lbm_initialize_fields): a dict of keyword arguments, or
    None for a strategy that is not a closed-form field (the Mei iteration)."""
    if isinstance(strategy, ZeroVelocityInitialCondition):
        return {}
    X, Y = node_grid(problem)
    cs = q.speed_of_sound_squared

    def sym(g):
        return (g[0, 0] + g[0, 0], g[0, 1] + g[1, 0], g[1, 1] + g[1, 1])

    if isinstance(strategy, (AnalyticalEquilibrium, AnalyticalEquilibriumAndOffEquilibrium)):
        out = {"rho": problem.density(q, X, Y, 0.0), "T": problem.pressure(q, X, Y) / problem.density(q, X, Y)}
        out["ux"], out["uy"] = lattice_velocity(q, problem, X, Y)
        if isinstance(strategy, AnalyticalEquilibriumAndOffEquilibrium):
            tau = cs * problem.lattice_viscosity()
            if isinstance(problem, TGV):  # analytical_offequilibrium.jl:50-87
                out["S"] = sym(problem.velocity_gradient(X, Y, 0.0))
                out["coef"], out["times_rho"] = -(cs * (tau + 0.5)) / 2, True
            else:  # analytical_offequilibrium.jl:10-49
                out["S"] = sym(problem.u_max ** 2 * problem.velocity_gradient(X, Y, 0.0))
                factor = problem.domain_size[0] * problem.domain_size[1]
                out["coef"] = -factor * 0.5 * ((tau + 0.5) * cs)
        return out
    if isinstance(strategy, (ConstantDensity, AnalyticalVelocityAndStress)):
        out = {}
        out["ux"], out["uy"] = lattice_velocity(q, problem, X, Y)
        if isinstance(strategy, AnalyticalVelocityAndStress):
            out["S"] = sym(problem.u_max ** 2 * problem.velocity_gradient(X, Y, 0.0))
            out["coef"] = -(cs * (cs * problem.lattice_viscosity() + 0.5)) / 2
        return out
    return None


def initialize(strategy, q, problem, cm=None):
    X, Y = node_grid(problem)
    shape = X.shape
    if isinstance(strategy, ZeroVelocityInitialCondition):
        return np.ascontiguousarray(np.broadcast_to(q.weights[:, None, None], (q.Q,) + shape), dtype=np.float64)
    if isinstance(strategy, (AnalyticalEquilibrium, AnalyticalEquilibriumAndOffEquilibrium)):
        rho = np.broadcast_to(problem.density(q, X, Y, 0.0), shape)
        u = lattice_velocity(q, problem, X, Y)
        T = np.broadcast_to(problem.pressure(q, X, Y) / problem.density(q, X, Y), shape)
        f = K.equilibrium(q, rho, u, T)
        if isinstance(strategy, AnalyticalEquilibriumAndOffEquilibrium):
            cs = q.speed_of_sound_squared
            if isinstance(problem, TGV):  # analytical_offequilibrium.jl:50-87
                g = problem.velocity_gradient(X, Y, 0.0)
                S = g + g.transpose(1, 0, *range(2, g.ndim))
                tau = cs * problem.lattice_viscosity()
                tau_eff = tau + 0.5
                for i in range(q.Q):
                    H = K.hermite(2, q.abscissae[:, i], q)
                    f[i] = f[i] - q.weights[i] * (((cs * tau_eff) * rho) * 1.0) / 2 * _dot_sym(H, S)
            else:  # analytical_offequilibrium.jl:10-49
                g = problem.u_max ** 2 * problem.velocity_gradient(X, Y, 0.0)
                S = g + g.transpose(1, 0, *range(2, g.ndim))
                tau = cs * problem.lattice_viscosity()
                factor = problem.domain_size[0] * problem.domain_size[1]
                for i in range(q.Q):
                    H = K.hermite(2, q.abscissae[:, i], q)
                    f[i] = f[i] + -factor * q.weights[i] * 0.5 * ((tau + 0.5) * cs) * _dot_sym(H, S)
        return np.ascontiguousarray(f)
    if isinstance(strategy, (ConstantDensity, AnalyticalVelocityAndStress)):
        u = lattice_velocity(q, problem, X, Y)
        f = K.equilibrium(q, np.ones(shape), u, np.ones(shape))
        if isinstance(strategy, AnalyticalVelocityAndStress):
            cs = q.speed_of_sound_squared
            g = problem.u_max ** 2 * problem.velocity_gradient(X, Y, 0.0)
            S = g + g.transpose(1, 0, *range(2, g.ndim))
            tau_eff = cs * problem.lattice_viscosity() + 0.5
            for i in range(q.Q):
                H = K.hermite(2, q.abscissae[:, i], q)
                f[i] = f[i] + -(q.weights[i] * (((cs * tau_eff) * 1.0) * 1.0) / 2 * _dot_sym(H, S))
        return np.ascontiguousarray(f)
    if isinstance(strategy, IterativeInitializationMeiEtAl):
        from .model import mei_initialize
        return mei_initialize(strategy, q, problem)
    if isinstance(strategy, AnalyticalVelocity):
        raise NotImplementedError("AnalyticalVelocity has no working initial condition in the reference")
    raise TypeError(f"unknown initialisation strategy {strategy!r}")
