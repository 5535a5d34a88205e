"""Processing methods (the reference's next!(pm, q, f, t) hook, L5) on top of the device
reductions of liblbm_gb300.

  TrackHydrodynamicErrors         processing_methods/track_hydrodynamic_errors.jl:1-242
  CompareWithAnalyticalSolution   processing_methods.jl:33-269
  ProcessIterativeInitialization  processing_methods/process_iterative_initialization.jl
  TakeSnapshots                   processing_methods/take_snapshots.jl:1-29 (no plotting)
  stop criteria                   processing_methods/stopping_criteria/*.jl

`pm.next(model, t)` has the reference's semantics (returns True to stop); `pm.df` holds the
same rows, as namedtuples with the reference's field names.  `pm.next_event(t)` tells the
time loop the first t' >= t at which next! does anything, so that the steps in between run
as one device batch.
"""
from __future__ import annotations

import collections
import math

import numpy as np

from . import _native as N
from .problems import (CouetteFlow, DecayingShearFlow, LidDrivenCavityFlow, PoiseuilleFlow, TaylorGreenVortex,
                       TGV, analytic_fields, problem_range)

TrackRow = collections.namedtuple(
    "TrackRow", ["timestep", "error_ρ", "error_u", "error_p", "error_σ_xx", "error_σ_xy", "error_σ_yy",
                 "error_σ_yx", "mass", "momentum", "energy"])
CompareRow = collections.namedtuple(
    "CompareRow", ["density", "momentum", "total_energy", "kinetic_energy", "internal_energy", "density_a",
                   "momentum_a", "total_energy_a", "kinetic_energy_a", "internal_energy_a", "error_u", "error_p",
                   "error_σ_xx", "error_σ_xy", "error_σ_yy", "error_σ_yx"])


def _div(a, b):
    """Julia Float64 division (x/0 -> ±Inf, 0/0 -> NaN) without Python exceptions."""
    with np.errstate(divide="ignore", invalid="ignore"):
        return float(np.float64(a) / np.float64(b))


def _sqrt(a):
    with np.errstate(invalid="ignore"):
        return float(np.sqrt(np.float64(a)))


# ---------------------------------------------------------------------------------------
# stop criteria
# ---------------------------------------------------------------------------------------
class StopCriteria:
    active = True
    reduce_kind = None  # the device reduction should_stop consumes (batched by simulate_batch)

    def should_stop(self, model) -> bool:
        return False


class NoStoppingCriteria(StopCriteria):
    active = False


class MeanVelocityStoppingCriteria(StopCriteria):
    """stopping_criteria.jl:20-72: stop when |ū_x / ū_x,old - 1| < tolerance, or on NaN."""
    reduce_kind = N.REDUCE_MEAN_VELOCITY

    def __init__(self, old_mean_velocity, tolerance, problem):
        self.old_mean_velocity = float(old_mean_velocity)
        self.tolerance = float(tolerance)
        self.problem = problem

    def should_stop(self, model) -> bool:
        s = model.lattice.reduce(N.REDUCE_MEAN_VELOCITY)
        u_mean = _div(s[0], s[1])
        converged = abs(_div(u_mean, self.old_mean_velocity) - 1)
        if converged < self.tolerance:
            return True
        if math.isnan(u_mean):
            return True
        self.old_mean_velocity = u_mean
        return False


class VelocityConvergenceStoppingCriteria(StopCriteria):
    """stopping_criteria.jl:74-132: √Σ|u - u_old|² / Σ|u_old|² < tolerance; the previous
    velocity field is kept on the device."""
    reduce_kind = N.REDUCE_VELOCITY_CONVERGENCE

    def __init__(self, tolerance, problem):
        self.tolerance = float(tolerance)
        self.problem = problem

    def should_stop(self, model) -> bool:
        s = model.lattice.reduce(N.REDUCE_VELOCITY_CONVERGENCE)
        converged = _div(_sqrt(s[0]), s[1])
        if converged < self.tolerance:
            return True
        if math.isnan(converged):
            return True
        return False


class DensityConvergence(StopCriteria):
    """density_convergence.jl:1-17.  Like the reference's `for x_idx in nx, y_idx in ny`
    loop it inspects the single node (nx, ny)."""

    def __init__(self, ϵ, nx, ny):
        self.ϵ = float(ϵ)
        self.nx, self.ny = int(nx), int(ny)
        self.ρ = 0.0
        self.ρ_old = 0.0

    def should_stop(self, model) -> bool:
        self.ρ_old = self.ρ
        self.ρ = model.lattice.density_at(self.nx - 1, self.ny - 1)
        dρ = abs(self.ρ - self.ρ_old)
        return dρ < self.ϵ or dρ > 100.0


def StopCriteriaFor(problem):
    """StopCriteria(problem) of the reference (stopping_criteria.jl:8-14)."""
    if isinstance(problem, PoiseuilleFlow):
        return MeanVelocityStoppingCriteria(0.0, 1e-12, problem)
    if isinstance(problem, CouetteFlow):
        return MeanVelocityStoppingCriteria(0.0, 1e-7, problem)
    if isinstance(problem, LidDrivenCavityFlow):
        return MeanVelocityStoppingCriteria(0.0, 1e-5, problem)
    if isinstance(problem, DecayingShearFlow):
        return MeanVelocityStoppingCriteria(0.0, 1e-8, problem) if problem.static else NoStoppingCriteria()
    return NoStoppingCriteria()


# ---------------------------------------------------------------------------------------
# processing methods
# ---------------------------------------------------------------------------------------
class ProcessingMethodBase:
    problem = None

    def next(self, model, t: int) -> bool:
        return False

    def next_event(self, t_from: int):
        """Smallest t >= t_from at which next() may act, or None."""
        return None

    def stop_reduction_due(self, t: int):
        """The device reduction kind next(model, t) will ask its stop criterion for, or None."""
        return None


class NoProcessing(ProcessingMethodBase):
    """A processing method that records nothing and never stops (pure stepping)."""

    def __init__(self, problem=None):
        self.problem = problem


def _events(t_from, should_process, stop_active, n_steps):
    if should_process:
        return t_from
    cands = []
    if stop_active:
        cands.append(((t_from + 99) // 100) * 100)
    if n_steps >= t_from:
        cands.append(n_steps)
    return min(cands) if cands else None


def _mass_scale(problem, nx, ny):
    _, _, xs, ys = problem_range(problem)
    D = ys * xs
    if nx == 1:
        D = ys
        if ny == 1:
            D = 1.0
    elif ny == 1:
        D = xs
    return D


class TrackHydrodynamicErrors(ProcessingMethodBase):
    def __init__(self, problem, should_process, n_steps, stop_criteria=None):
        self.problem = problem
        self.should_process = bool(should_process)
        self.n_steps = int(n_steps)
        self.stop_criteria = StopCriteriaFor(problem) if stop_criteria is None else stop_criteria
        self.df = []

    def next_event(self, t_from):
        return _events(t_from, self.should_process, self.stop_criteria.active, self.n_steps)

    def stop_reduction_due(self, t):
        return self.stop_criteria.reduce_kind if t % 100 == 0 else None

    def next(self, model, t):
        should_stop = False
        if t % 100 == 0 and self.stop_criteria.should_stop(model):
            should_stop = True
        if not should_stop and t != self.n_steps and not self.should_process:
            return False
        self.df.append(track_errors(model, self.problem, t))
        return should_stop


def track_inputs(model, problem, t):
    """The inputs of the TRACK_ERRORS reduction at step t: (analytic fields, tau, u_max, area)."""
    q = model.quadrature
    fields = analytic_fields(q, problem, t * problem.delta_t())
    return fields, q.speed_of_sound_squared * problem.lattice_viscosity(), problem.u_max, 0.0


def track_errors(model, problem, t):
    """One TrackHydrodynamicErrors row for the model's current state at step t
    (track_hydrodynamic_errors.jl:68-221) from one device reduction (or the sums a batched
    reduction already supplied)."""
    if N.REDUCE_TRACK_ERRORS in model.lattice.prefetched:
        s = model.lattice.reduce(N.REDUCE_TRACK_ERRORS)
    else:
        fields, tau, u_max, _ = track_inputs(model, problem, t)
        s = model.lattice.reduce(N.REDUCE_TRACK_ERRORS, fields, tau=tau, u_max=u_max)
    D_ = _mass_scale(problem, model.lattice.nx, model.lattice.ny)
    return TrackRow(int(t), _sqrt(s[0]), _sqrt(_div(s[1], s[7])), _sqrt(_div(s[2], s[12])),
                    _sqrt(_div(s[3], s[8])), _sqrt(_div(s[4], s[10])), _sqrt(_div(s[5], s[9])),
                    _sqrt(_div(s[6], s[11])), D_ * s[13], D_ * s[14], D_ * s[15])


class CompareWithAnalyticalSolution(ProcessingMethodBase):
    def __init__(self, problem, should_process, n_steps, stop_criteria=None):
        self.problem = problem
        self.should_process = bool(should_process)
        self.n_steps = int(n_steps)
        self.stop_criteria = StopCriteriaFor(problem) if stop_criteria is None else stop_criteria
        self.df = []

    def next_event(self, t_from):
        return _events(t_from, self.should_process, self.stop_criteria.active, self.n_steps)

    def stop_reduction_due(self, t):
        return self.stop_criteria.reduce_kind if t % 100 == 0 else None

    def next(self, model, t):
        if t % 100 == 0 and self.stop_criteria.should_stop(model):
            self.df.append(compare_process(model, self.problem, t * self.problem.delta_t()))
            return True
        if not self.should_process and t != self.n_steps:
            return False
        self.df.append(compare_process(model, self.problem, t * self.problem.delta_t()))
        return False


def compare_inputs(model, problem, time):
    """The inputs of the COMPARE reduction at physical time `time`: (fields, tau, u_max, area)."""
    _, _, xs, ys = problem_range(problem)
    return analytic_fields(model.quadrature, problem, time), 0.0, problem.u_max, ys * xs


def compare_process(model, problem, time):
    """process!(problem, q, f, time, stats) (processing_methods.jl:142-269)."""
    if N.REDUCE_COMPARE in model.lattice.prefetched:
        s = model.lattice.reduce(N.REDUCE_COMPARE)
    else:
        fields, _, u_max, area = compare_inputs(model, problem, time)
        s = model.lattice.reduce(N.REDUCE_COMPARE, fields, u_max=u_max, area=area)
    return CompareRow(s[0], s[1], s[2], s[3], s[4], s[5], s[6], s[7], s[8], s[9], _sqrt(s[10]), _sqrt(s[11]),
                      0.0, 0.0, 0.0, 0.0)


class ProcessIterativeInitialization(ProcessingMethodBase):
    """Stops when DensityConvergence trips (process_iterative_initialization.jl:1-24); it has
    no problem field, so the time loop runs with Δt = 0."""

    def __init__(self, ϵ, problem, process_method=None):
        self.stop_criteria = DensityConvergence(ϵ, problem.NX, problem.NY)
        self.internal_process_method = process_method
        self.n_steps = 100
        self.problem = None

    def next_event(self, t_from):
        return t_from

    def next(self, model, t):
        return self.stop_criteria.should_stop(model)


class TakeSnapshots(ProcessingMethodBase):
    """Copies f_stream at every `every_t`-th step, or at the listed steps (take_snapshots.jl:12-29)."""

    def __init__(self, problem, every_t):
        self.problem = problem
        self.every_t = every_t
        self.snapshots = []
        self.timesteps = []

    def next_event(self, t_from):
        if isinstance(self.every_t, int):
            return ((t_from + self.every_t - 1) // self.every_t) * self.every_t
        later = [t for t in self.every_t if t >= t_from]
        return min(later) if later else None

    def next(self, model, t):
        if isinstance(self.every_t, int) and t % self.every_t != 0:
            return False
        if not isinstance(self.every_t, int) and t not in self.every_t:
            return False
        self.snapshots.append(model.f_stream)
        self.timesteps.append(t)
        return False


def ProcessingMethod(problem, should_process, n_steps, stop_criteria=None):
    """Factory of the reference (processing_methods.jl:10-29)."""
    if isinstance(problem, (TaylorGreenVortex, DecayingShearFlow, TGV)):
        return TrackHydrodynamicErrors(problem, should_process, n_steps, stop_criteria)
    return CompareWithAnalyticalSolution(problem, should_process, n_steps, stop_criteria)
