"""Collision models of LatticeBoltzmann.jl, as descriptors for the fused device kernel.

  SRT(τ[, force])                     srt.jl:1-16
  TRT(τ_a, τ_s)  -- note the order:   trt.jl:6 (the two-argument form swaps to (τ_s, τ_a))
  TRT.fields(τ_s, τ_a, force)         the struct's positional constructor, trt.jl:1-5
  TRT_Λ(Λ)                            magic-parameter factory, trt.jl:24-40
  MRT(q, τ[, force]) / MRT(q, τ_s, τ_a[, force]) / MRT(q, τs[, force])   mrt.jl:1-47
      (like the reference, the scalar and two-τ constructors drop the force)
  CollisionModel(cm, q, problem)      collision_models.jl:11-18 and the per-model factories

A `force` is either None or "problem": the problem's lattice_force(problem, x, y, t), as the
reference's closures `(x_idx, y_idx, t) -> lattice_force(problem, x_idx, y_idx, t)` are.
A problem must be attached (model construction does this) to evaluate it.
"""
from __future__ import annotations

from .quadratures import Quadrature, order


class CollisionModel:
    force = None

    def __init__(self, *a, **k):  # the factory function below carries the reference's name
        raise TypeError("use SRT, TRT, MRT or the CollisionModel(cm, q, problem) factory")


class SRT(CollisionModel):
    def __init__(self, τ, force=None):
        self.τ = float(τ)
        self.force = force

    def __repr__(self):
        return f"SRT({self.τ})"


class TRT(CollisionModel):
    def __init__(self, τ_a, τ_s):
        # TRT(τ_a, τ_s) = TRT(τ_s, τ_a, nothing)  (trt.jl:6)
        self.τ_symmetric = float(τ_s)
        self.τ_asymmetric = float(τ_a)
        self.force = None

    @classmethod
    def fields(cls, τ_symmetric, τ_asymmetric, force=None):
        m = cls.__new__(cls)
        m.τ_symmetric = float(τ_symmetric)
        m.τ_asymmetric = float(τ_asymmetric)
        m.force = force
        return m

    def __repr__(self):
        return f"TRT(τ_s={self.τ_symmetric}, τ_a={self.τ_asymmetric})"


class TRT_Λ:
    """Factory for a TRT operator with magic parameter Λ: τ_a = ½ + Λ / (τ_s - ½)."""

    def __init__(self, Λ):
        self.Λ = float(Λ)


class MRT(CollisionModel):
    def __init__(self, q: Quadrature, τ, τ_a=None, force=None):
        N = int(round(order(q) / 2))  # Julia round(Int, ·) rounds half to even, as Python does
        if isinstance(τ, (list, tuple)):
            self.τs = [float(t) for t in τ]
            self.force = force  # only the vector form keeps the force (mrt.jl:29-34)
        elif τ_a is None or not isinstance(τ_a, (int, float)):
            self.τs = [float(τ)] * N
            self.force = None   # MRT(q, τ, force) drops it (mrt.jl:19-22)
        else:
            self.τs = ([float(τ), float(τ_a)] * N)[:N]
            self.force = None   # MRT(q, τ_s, τ_a, force) drops it (mrt.jl:24-27)

    def __repr__(self):
        return f"MRT(τs={self.τs})"


class IterativeInitializationCollisionModel(CollisionModel):
    """Fixed-velocity BGK of the Mei et al. iterative initialisation
    (iterative_initialization.jl:1-60); the nonlinear term is built by the model."""

    def __init__(self, τ):
        self.τ = float(τ)
        self.force = None


def _factory_tau(q, problem):
    return q.speed_of_sound_squared * problem.lattice_viscosity() + 0.5


def make_collision_model(cm, q: Quadrature, problem):
    """CollisionModel(cm, q, problem): instances pass through; types build the default
    operator for the problem (srt.jl:7-16, trt.jl:8-21, mrt.jl:36-47, collision_models.jl:11-18)."""
    if isinstance(cm, CollisionModel):
        return cm
    force = "problem" if problem.has_external_force() else None
    if isinstance(cm, TRT_Λ) or cm is TRT:
        Λ = cm.Λ if isinstance(cm, TRT_Λ) else 1 / 4
        τ = _factory_tau(q, problem)
        τ_ = 0.5 + Λ / (τ - 0.5)
        return TRT.fields(τ, τ_, force)
    if cm is MRT:
        τ = _factory_tau(q, problem)
        m = MRT(q, [τ] * order(q))
        m.force = force
        return m
    # SRT and the default for any other type
    return SRT(_factory_tau(q, problem), force)
