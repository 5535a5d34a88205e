"""Gradients of a field loss through the lattice-Boltzmann time loop (lbm_adjoint_*).

The reference has no differentiation (no ForwardDiff / ChainRulesCore in its manifests, and its
SRT hard-types τ as Float64).  This module exposes the discrete adjoint of the device kernels for
D2Q9 / D2Q13 lattices with SRT, TRT or regularised MRT, a uniform force and bounce-back /
moving-wall boundaries:

    L(u0, τ, F) = Σ_x |u(f_T) - u*|²,   f_0 = f_eq(1, u0),   f_{t+1} = apply!(stream(collide(f_t; τ, F))),

`AdjointProblem.run(u0, u_target)` returns L, ∂L/∂τ_s, ∂L/∂τ_a, ∂L/∂F and ∂L/∂u0 (MRT: "dtau_s" is
∂L/∂τ_2, the second-order relaxation time, which also scales the force shift; "dtau_a" is 0) (binomial
checkpointing with a given number of state slots, one CUDA graph).  `LBMLoss` wraps it as a torch.autograd.Function, the Python
counterpart of a ChainRulesCore.rrule for `simulate`.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _native as N
from .device import DeviceLattice


class AdjointProblem:
    """The adjoint of `nsteps` steps of an nx x ny lattice.  `boundary_conditions` are BounceBack /
    MovingWall instances (applied in list order after the stream, as in the forward model);
    `slots` is the number of lattice states kept for the binomial checkpointing schedule (0: the
    fewest with which no step is recomputed more than twice)."""

    def __init__(self, q, nx, ny, collision_model, force=(0.0, 0.0), nsteps=100, slots=0, storage="f64",
                 boundary_conditions=()):
        self.q, self.nx, self.ny, self.nsteps = q, int(nx), int(ny), int(nsteps)
        self.collision_model = collision_model
        self.force = (float(force[0]), float(force[1]))
        dev_force = ("constant", self.force) if any(self.force) else None
        self.lattice = DeviceLattice(q, nx, ny, collision_model, tuple(boundary_conditions), force=dev_force,
                                     storage=storage)
        h = C.c_void_p()
        st = N.lib().lbm_adjoint_create(C.byref(h), self.lattice.h, self.nsteps, int(slots))
        if st != N.LBM_OK:
            raise N.LbmError(st, N.lib().lbm_last_error(self.lattice.h).decode())
        self.h = h

    def info(self):
        """{"slots", "forward_steps", "device_bytes"} of the checkpointing schedule."""
        a, b, c = C.c_int64(), C.c_int64(), C.c_int64()
        N.check(None, N.lib().lbm_adjoint_info(self.h, C.byref(a), C.byref(b), C.byref(c)))
        return {"slots": a.value, "forward_steps": b.value, "device_bytes": c.value}

    def run(self, u0, u_target, want_grad_u0=True):
        """u0, u_target: arrays of shape (2, NY, NX).  Returns a dict with the loss and gradients."""
        if not getattr(self, "h", None):
            raise ValueError("the adjoint problem is closed")
        u0 = np.ascontiguousarray(u0, dtype=np.float64)
        ut = np.ascontiguousarray(u_target, dtype=np.float64)
        if u0.shape != (2, self.ny, self.nx) or ut.shape != u0.shape:
            raise ValueError(f"u0 and u_target must have shape (2, {self.ny}, {self.nx}), "
                             f"got {u0.shape} and {ut.shape}")
        res = np.zeros(8)
        g = np.zeros_like(u0) if want_grad_u0 else None
        st = N.lib().lbm_adjoint_run(self.h, u0.ctypes.data_as(N._DP), ut.ctypes.data_as(N._DP),
                                     res.ctypes.data_as(N._DP), g.ctypes.data_as(N._DP) if g is not None else None)
        if st != N.LBM_OK:
            raise N.LbmError(st, N.lib().lbm_adjoint_last_error(self.h).decode())
        out = {"loss": res[0], "dtau_s": res[1], "dtau_a": res[2], "dF": np.array(res[3:5])}
        if g is not None:
            out["grad_u0"] = g
        return out

    def loss(self, u0, u_target):
        return self.run(u0, u_target, want_grad_u0=False)["loss"]

    def close(self):
        if getattr(self, "h", None):
            N.lib().lbm_adjoint_destroy(self.h)
            self.h = None
        self.lattice.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def trt_magic(tau_s, Λ=0.25):
    """τ_a of the TRT magic-parameter relation τ_a = ½ + Λ / (τ_s - ½) (trt.jl:14-15)."""
    return 0.5 + Λ / (tau_s - 0.5)


def magic_total_derivative(res, tau_s, Λ=0.25):
    """dL/dτ_s along the magic relation: ∂L/∂τ_s + ∂L/∂τ_a · dτ_a/dτ_s."""
    return res["dtau_s"] + res["dtau_a"] * (-Λ / (tau_s - 0.5) ** 2)


def divergence_free_field(nx, ny, kmax=8, amplitude=0.01, seed=0):
    """u = (∂ψ/∂y, -∂ψ/∂x) of a stream function ψ = Σ_{0<|k|≤kmax} a_k cos(k·x) + b_k sin(k·x) with
    seeded Gaussian a, b, scaled to max|u| = amplitude; shape (2, NY, NX)."""
    rng = np.random.default_rng(seed)
    X, Y = np.meshgrid(np.arange(nx), np.arange(ny))
    ux = np.zeros((ny, nx))
    uy = np.zeros((ny, nx))
    for kx in range(-kmax, kmax + 1):
        for ky in range(-kmax, kmax + 1):
            if (kx == 0 and ky == 0) or kx * kx + ky * ky > kmax * kmax:
                continue
            a, b = rng.normal(size=2)
            px, py = 2 * math.pi * kx / nx, 2 * math.pi * ky / ny
            ph = px * X + py * Y
            # ψ = a cos(ph) + b sin(ph);  u = ∂ψ/∂y, v = -∂ψ/∂x
            dpsi = -a * np.sin(ph) + b * np.cos(ph)
            ux += py * dpsi
            uy -= px * dpsi
    s = amplitude / max(np.max(np.hypot(ux, uy)), 1e-300)
    return np.stack([ux * s, uy * s])


try:
    import torch

    class LBMLoss(torch.autograd.Function):
        """L(u0, τ_s, F) with the adjoint as backward (the rrule of `simulate` for this loss)."""

        @staticmethod
        def forward(ctx, u0, tau_s, force, problem_factory, u_target):
            tau = float(tau_s)
            F = (float(force[0]), float(force[1]))
            prob = problem_factory(tau, F)
            res = prob.run(u0.detach().cpu().numpy(), u_target)
            prob.close()
            ctx.save_for_backward(torch.tensor(res["grad_u0"]), torch.tensor(magic_total_derivative(res, tau)),
                                  torch.tensor(res["dF"]))
            return torch.tensor(res["loss"], dtype=torch.float64)

        @staticmethod
        def backward(ctx, gout):
            gu, gt, gf = ctx.saved_tensors
            return gout * gu, gout * gt, gout * gf, None, None
except Exception:  # torch is optional for the module itself
    LBMLoss = None
