"""Python handle on the CPU oracle (``oracle/lbm_oracle.cpp``).

TEST INFRASTRUCTURE ONLY: the test-suite, the smoke check and the CPU-baseline leg of the
benchmark use this module as the oracle of the CUDA path.  Nothing in the product imports
it.

Arrays follow the reference's Julia layout ``f[x, y, i]`` (column-major), which is the
C-contiguous numpy shape ``(Q, ny, nx)``: ``f[i, y, x] == f_julia[x+1, y+1, i+1]``.

Problem constructors below restate the reference's keyword defaults and size overrides
(the file:line of each is given) so that tests build the same inputs the reference would.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SO = os.path.join(_HERE, "_build", "liblbm_oracle.so")
_lock = threading.Lock()
_lib = None

QUAD_IDS = {"D2Q4": 0, "D2Q5": 1, "D2Q9": 2, "D2Q13": 3, "D2Q17": 4, "D2Q21": 5, "D2Q37": 6}

P_TAYLOR_GREEN, P_TGV, P_POISEUILLE, P_COUETTE, P_DECAYING_SHEAR = 0, 1, 2, 3, 4
P_LID_DRIVEN, P_LIN_THERMAL, P_LIN_SHEAR, P_INIT_TEST, P_SHEAR_WAVE = 5, 6, 7, 8, 9

INIT_ZERO_VELOCITY, INIT_EQUILIBRIUM, INIT_EQ_OFFEQ, INIT_CONSTANT_DENSITY, INIT_VELOCITY_STRESS = 0, 1, 2, 3, 4

PM_TRACK, PM_COMPARE, PM_ITERATIVE, PM_NONE = 0, 1, 2, 3
STOP_NONE, STOP_MEAN_VELOCITY, STOP_VELOCITY, STOP_DENSITY = 0, 1, 2, 3


class OrcProblem(C.Structure):
    _fields_ = [("kind", C.c_int), ("nx", C.c_int), ("ny", C.c_int), ("is_static", C.c_int),
                ("rho_0", C.c_double), ("u_max", C.c_double), ("nu", C.c_double),
                ("dom0", C.c_double), ("dom1", C.c_double),
                ("A", C.c_double), ("B", C.c_double), ("a", C.c_double), ("b", C.c_double),
                ("k_x", C.c_double), ("k_y", C.c_double), ("G", C.c_double), ("k", C.c_double),
                ("u_0", C.c_double), ("tau", C.c_double),
                ("theta_0", C.c_double), ("rho_t", C.c_double), ("u_t", C.c_double),
                ("kappa", C.c_double), ("q_cs", C.c_double)]


class OrcCollision(C.Structure):
    _fields_ = [("kind", C.c_int), ("tau", C.c_double * 8), ("ntau", C.c_int), ("force_kind", C.c_int)]


class OrcBC(C.Structure):
    _fields_ = [("kind", C.c_int), ("direction", C.c_int), ("x_lo", C.c_int), ("x_hi", C.c_int),
                ("y_lo", C.c_int), ("y_hi", C.c_int), ("u", C.c_double * 2), ("rho", C.c_double),
                ("T", C.c_double)]


class OrcProcessing(C.Structure):
    _fields_ = [("pm_kind", C.c_int), ("should_process", C.c_int), ("n_steps", C.c_long),
                ("stop_kind", C.c_int), ("stop_tol", C.c_double), ("has_problem", C.c_int),
                ("nthreads", C.c_int)]


class OrcRow(C.Structure):
    _fields_ = [("timestep", C.c_long), ("v", C.c_double * 16)]


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (g++, OpenMP) unless it is already built."""
    with _lock:
        if force or not os.path.exists(_SO) or \
                os.path.getmtime(_SO) < os.path.getmtime(os.path.join(_HERE, "lbm_oracle.cpp")):
            subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _SO


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_SO)
        dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
        ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
        L.orc_quadrature.argtypes = [C.c_int, C.POINTER(C.c_int), ip, ip, dp, C.POINTER(C.c_double),
                                     C.POINTER(C.c_int), ip]
        L.orc_hermite.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, dp]
        L.orc_equilibrium.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, dp]
        L.orc_hermite_equilibrium.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, dp]
        L.orc_moments.argtypes = [C.c_int, dp, C.c_double, dp]
        L.orc_problem_fields.argtypes = [C.POINTER(OrcProblem), C.c_int, C.c_double, dp]
        L.orc_problem_scalars.argtypes = [C.POINTER(OrcProblem), dp]
        L.orc_problem_coords.argtypes = [C.POINTER(OrcProblem), dp, dp]
        L.orc_force_field.argtypes = [C.POINTER(OrcProblem), C.c_double, dp]
        L.orc_initialize.argtypes = [C.c_int, C.c_int, C.POINTER(OrcProblem), dp]
        L.orc_collide.argtypes = [C.c_int, C.POINTER(OrcProblem), C.POINTER(OrcCollision), C.c_int, C.c_int,
                                  dp, dp, C.c_double]
        L.orc_stream.argtypes = [C.c_int, C.c_int, C.c_int, dp, dp]
        L.orc_apply_bcs.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(OrcBC), dp, dp]
        L.orc_track_errors.argtypes = [C.c_int, C.POINTER(OrcProblem), dp, C.c_long, dp]
        L.orc_simulate.argtypes = [C.c_int, C.POINTER(OrcProblem), C.POINTER(OrcCollision), C.c_int,
                                   C.POINTER(OrcBC), C.POINTER(OrcProcessing), C.c_long, C.c_long, dp,
                                   C.POINTER(OrcRow), C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_long)]
        L.orc_run.argtypes = [C.c_int, C.POINTER(OrcProblem), C.POINTER(OrcCollision), C.c_int,
                              C.POINTER(OrcBC), C.c_long, C.c_long, C.c_double, C.c_int, dp]
        L.orc_tangent_loss.argtypes = [C.c_int, C.c_int, dp, dp, C.c_int, C.c_int, dp, dp, dp, C.c_void_p,
                                       C.c_long, C.c_int, C.c_void_p, C.c_int, dp]
        L.orc_tangent_loss.restype = C.c_int
        L.orc_max_threads.restype = C.c_int
        _lib = L
    return _lib


def qid(q) -> int:
    return QUAD_IDS[q] if isinstance(q, str) else int(q)


# ----------------------------------------------------------------------------------------
# quadratures and per-node kinetics
# ----------------------------------------------------------------------------------------
def quadrature(q):
    Q = C.c_int()
    cx = np.zeros(37, np.int32)
    cy = np.zeros(37, np.int32)
    w = np.zeros(37)
    opp = np.zeros(37, np.int32)
    cs = C.c_double()
    order = C.c_int()
    rc = lib().orc_quadrature(qid(q), C.byref(Q), cx, cy, w, C.byref(cs), C.byref(order), opp)
    assert rc == 0
    n = Q.value
    return {"Q": n, "cx": cx[:n].copy(), "cy": cy[:n].copy(), "w": w[:n].copy(), "cs": cs.value,
            "order": order.value, "opposite": opp[:n].copy()}


def hermite(q, n, xi):
    H = np.zeros(16)
    lib().orc_hermite(qid(q), n, int(xi[0]), int(xi[1]), H)
    return H[: 1 << n]


def equilibrium(q, rho, u):
    f = np.zeros(37)
    lib().orc_equilibrium(qid(q), rho, u[0], u[1], f)
    return f[: quadrature(q)["Q"]]


def hermite_equilibrium(q, rho, u, T=1.0):
    f = np.zeros(37)
    lib().orc_hermite_equilibrium(qid(q), rho, u[0], u[1], T, f)
    return f[: quadrature(q)["Q"]]


def moments(q, f, tau=1.0):
    """ρ, ux, uy, pressure, temperature, σ (column-major 2x2) of one node's populations."""
    out = np.zeros(9)
    lib().orc_moments(qid(q), np.ascontiguousarray(f, dtype=np.float64), tau, out)
    return out


# ----------------------------------------------------------------------------------------
# problems: constructors mirror the reference's defaults
# ----------------------------------------------------------------------------------------
def _problem(kind, nx, ny, **kw):
    p = OrcProblem()
    p.kind, p.nx, p.ny = kind, int(nx), int(ny)
    p.rho_0, p.dom0, p.dom1 = 1.0, 1.0, 1.0
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def taylor_green_vortex(nu=1.0 / 6.0, scale=2, NX=None, NY=None, domain=(2 * math.pi, 2 * math.pi),
                        static=True, A=1.0, B=-1.0, a=1.0, b=1.0):
    """TaylorGreenVortex(ν, scale, NX, NY, domain; static, A, B, a, b): taylor_green_vortex.jl:14-34."""
    NX = 16 * scale if NX is None else NX
    NY = NX if NY is None else NY
    return _problem(P_TAYLOR_GREEN, NX, NY, u_max=0.01 / scale, nu=nu, dom0=domain[0], dom1=domain[1],
                    is_static=int(static), A=A, B=B, a=a, b=b)


def tgv(q, tau, scale=2, NX=None, NY=None, u_max=None):
    """TGV(q, τ, scale, NX, NY, u_max): second_order_convergence.jl:13-26 (u_max is stored as u_0)."""
    NX = 16 * scale if NX is None else NX
    NY = NX if NY is None else NY
    u0 = 0.02 / scale if u_max is None else u_max
    cs = quadrature(q)["cs"]
    nu = (tau - 0.5) / cs
    return _problem(P_TGV, NX, NY, u_max=1.0, u_0=u0, tau=tau, nu=nu, q_cs=cs, is_static=0)


def poiseuille(nu=1.0 / 6.0, scale=2, NX=None, NY=None, domain=(1.0, 1.0)):
    """PoiseuilleFlow(ν, scale, NX, NY, domain): poiseuille.jl:12-26 (NX forced to 3)."""
    NX = 5 * scale if NX is None else NX
    NY = NX if NY is None else NY
    return _problem(P_POISEUILLE, 3, NY, u_max=0.1 / scale, nu=nu, dom0=domain[0], dom1=domain[1],
                    k=1.0, G=1.0)


def poiseuille_struct(rho_0, u_max, nu, NX, NY, k, domain, G):
    """Positional PoiseuilleFlow(ρ0, u_max, ν, NX, NY, k, domain, G): poiseuille.jl:1-10."""
    return _problem(P_POISEUILLE, NX, NY, rho_0=rho_0, u_max=u_max, nu=nu, dom0=domain[0],
                    dom1=domain[1], k=k, G=G)


def couette(nu=1.0 / 6.0, scale=2, NX=None, NY=None, domain=(1.0, 1.0)):
    """CouetteFlow(ν, scale, NX, NY, domain): couette_flow.jl:10-25 (NX forced to 1)."""
    NX = 5 * scale if NX is None else NX
    NY = NX if NY is None else NY
    return _problem(P_COUETTE, 1, NY, u_max=0.01 / scale, nu=nu, dom0=domain[0], dom1=domain[1])


def decaying_shear_flow(nu=1.0 / 6.0, scale=2, NX=None, NY=None, domain=(2 * math.pi, 2 * math.pi),
                        static=True, A=1.0, B=1.0, k_x=1.0, k_y=0.0):
    """DecayingShearFlow(ν, scale, NX, NY, domain; static, A, B, k_x, k_y): decaying_shear_flow.jl:14-36."""
    NX = 8 * scale if NX is None else NX
    NY = NX if NY is None else NY
    if k_y == 0.0:
        NY = 3
    if k_x == 0.0:
        NX = 3
    return _problem(P_DECAYING_SHEAR, NX, NY, u_max=0.02 / scale, nu=nu, dom0=domain[0], dom1=domain[1],
                    is_static=int(static), A=A, B=B, k_x=k_x, k_y=k_y)


def lid_driven_cavity(nu=1.0 / 6.0, scale=2, NX=None, NY=None, domain=(1.0, 1.0)):
    """LidDrivenCavityFlow(ν, scale, NX, NY, domain): lid_driven_cavity.jl:10-23."""
    NX = 16 * scale if NX is None else NX
    NY = NX if NY is None else NY
    return _problem(P_LID_DRIVEN, NX, NY, u_max=0.01 / scale, nu=nu, dom0=domain[0], dom1=domain[1])


def init_test_problem(N=4, nu=1.0 / 6.0):
    """InitializationTestProblem(N, ν) of the reference's tests: test/initial_conditions.jl:12-26."""
    return _problem(P_INIT_TEST, N, N, u_max=1.0, nu=nu)


def shear_wave(nx, ny, nu, u0=0.01):
    """Lattice-unit shear wave u_x = u0 sin(2π y / Ny), ρ = 1, Δx = Δt = 1."""
    return _problem(P_SHEAR_WAVE, nx, ny, u_max=1.0, u_0=u0, nu=nu, dom0=float(nx), dom1=float(ny))


def problem_scalars(p):
    out = np.zeros(5)
    lib().orc_problem_scalars(C.byref(p), out)
    return {"delta_x": out[0], "delta_t": out[1], "viscosity": out[2], "x_step": out[3], "y_step": out[4]}


def problem_coords(p):
    xr = np.zeros(p.nx)
    yr = np.zeros(p.ny)
    lib().orc_problem_coords(C.byref(p), xr, yr)
    return xr, yr


def problem_fields(p, q, t):
    """Analytic ρ, ux, uy, p, σ(col-major) fields at physical time t, shape (9, ny, nx)."""
    out = np.zeros((9, p.ny, p.nx))
    lib().orc_problem_fields(C.byref(p), qid(q), t, out)
    return out


def force_field(p, t=0.0):
    out = np.zeros((2, p.ny, p.nx))
    lib().orc_force_field(C.byref(p), t, out)
    return out


def initialize(strategy, q, p):
    Q = quadrature(q)["Q"]
    f = np.zeros((Q, p.ny, p.nx))
    rc = lib().orc_initialize(int(strategy), qid(q), C.byref(p), f)
    if rc != 0:
        raise ValueError("unsupported initialisation strategy")
    return f


# ----------------------------------------------------------------------------------------
# collision models, BCs, time loop
# ----------------------------------------------------------------------------------------
def collision(kind, taus, force=False):
    """kind: 'SRT' (τ), 'TRT' (τ_s, τ_a), 'MRT' (τ_1..τ_N), 'ITER' (τ)."""
    cm = OrcCollision()
    cm.kind = {"SRT": 0, "TRT": 1, "MRT": 2, "ITER": 3}[kind]
    taus = list(taus)
    for k, t in enumerate(taus):
        cm.tau[k] = t
    cm.ntau = len(taus)
    cm.force_kind = int(bool(force))
    return cm


def bc(kind, direction, xs, ys, u=(0.0, 0.0), rho=1.0, T=1.0):
    """kind 'bounce_back' | 'moving_wall'; direction 'north' | 'east' | 'south' | 'west';
    xs, ys 1-based inclusive (lo, hi) ranges as in the reference's BounceBack(dir, 1:NX, 1:NY)."""
    b = OrcBC()
    b.kind = {"bounce_back": 0, "moving_wall": 1}[kind]
    b.direction = {"north": 0, "east": 1, "south": 2, "west": 3}[direction]
    b.x_lo, b.x_hi = xs
    b.y_lo, b.y_hi = ys
    b.u[0], b.u[1] = float(u[0]), float(u[1])
    b.rho, b.T = rho, T
    return b


def _bc_array(bcs):
    arr = (OrcBC * max(1, len(bcs)))()
    for k, b in enumerate(bcs):
        arr[k] = b
    return arr


def collide(q, f, cm, problem=None, time=0.0):
    f = np.ascontiguousarray(f, dtype=np.float64)
    _, ny, nx = f.shape
    p = problem if problem is not None else _problem(P_LID_DRIVEN, nx, ny)
    out = np.empty_like(f)
    lib().orc_collide(qid(q), C.byref(p), C.byref(cm), nx, ny, f, out, time)
    return out


def stream(q, f):
    f = np.ascontiguousarray(f, dtype=np.float64)
    _, ny, nx = f.shape
    out = np.empty_like(f)
    lib().orc_stream(qid(q), nx, ny, f, out)
    return out


def apply_bcs(q, bcs, f_new, f_old):
    f_new = np.ascontiguousarray(f_new, dtype=np.float64).copy()
    f_old = np.ascontiguousarray(f_old, dtype=np.float64)
    _, ny, nx = f_new.shape
    lib().orc_apply_bcs(qid(q), nx, ny, len(bcs), _bc_array(bcs), f_new, f_old)
    return f_new


def track_errors(q, p, f, t):
    out = np.zeros(10)
    lib().orc_track_errors(qid(q), C.byref(p), np.ascontiguousarray(f, dtype=np.float64), int(t), out)
    keys = ["error_rho", "error_u", "error_p", "error_sigma_xx", "error_sigma_xy", "error_sigma_yy",
            "error_sigma_yx", "mass", "momentum", "energy"]
    return dict(zip(keys, out))


TRACK_KEYS = ["error_rho", "error_u", "error_p", "error_sigma_xx", "error_sigma_xy", "error_sigma_yy",
              "error_sigma_yx", "mass", "momentum", "energy"]
COMPARE_KEYS = ["density", "momentum", "total_energy", "kinetic_energy", "internal_energy", "density_a",
                "momentum_a", "total_energy_a", "kinetic_energy_a", "internal_energy_a", "error_u",
                "error_p"]


def simulate(q, p, cm, bcs, f0, t_first, t_last, pm_kind=PM_TRACK, should_process=False, n_steps=None,
             stop_kind=STOP_NONE, stop_tol=0.0, has_problem=True, nthreads=1, max_rows=100000):
    """simulate(model, t_first:t_last) with a processing method; returns (f, rows, stopped_at)."""
    f = np.ascontiguousarray(f0, dtype=np.float64).copy()
    pm = OrcProcessing()
    pm.pm_kind, pm.should_process = pm_kind, int(should_process)
    pm.n_steps = t_last if n_steps is None else n_steps
    pm.stop_kind, pm.stop_tol, pm.has_problem, pm.nthreads = stop_kind, stop_tol, int(has_problem), nthreads
    rows = (OrcRow * max_rows)()
    nrows = C.c_int()
    stopped = C.c_long()
    lib().orc_simulate(qid(q), C.byref(p), C.byref(cm), len(bcs), _bc_array(bcs), C.byref(pm), t_first,
                       t_last, f, rows, max_rows, C.byref(nrows), C.byref(stopped))
    keys = TRACK_KEYS if pm_kind == PM_TRACK else COMPARE_KEYS
    out = []
    for k in range(min(nrows.value, max_rows)):
        r = {"timestep": rows[k].timestep}
        r.update({kk: rows[k].v[j] for j, kk in enumerate(keys)})
        out.append(r)
    return f, out, (stopped.value if stopped.value >= 0 else None)


def run(q, p, cm, bcs, f0, t_first, t_last, dt=0.0, nthreads=1):
    """The bare collide → stream → BC loop for t in t_first:t_last (CPU baseline workload)."""
    f = np.ascontiguousarray(f0, dtype=np.float64).copy()
    lib().orc_run(qid(q), C.byref(p), C.byref(cm), len(bcs), _bc_array(bcs), t_first, t_last, dt,
                  nthreads, f)
    return f


def tangent_loss(q, kind, taus, F, u0, ut, nsteps, seed=(0.0, 0.0, 0.0, 0.0), du0=None, nthreads=1, bcs=()):
    """L = Σ |u(f_T) - ut|² after `nsteps` collide → periodic stream → apply!(bcs) steps from
    f_0 = equilibrium(1, u0) (SRT `kind` "SRT" with τ = taus[0], TRT with τ_s, τ_a = taus, MRT of a
    second-order set with τs[1], τs[2] = taus (the outputs depend on τs[2] only), uniform
    lattice force F, the boundary conditions `bcs` built by bc()), and its forward-mode derivative
    along seed = (dτ_0, dτ_1, dF_x, dF_y) and the u0 direction du0, propagated with dual numbers.
    u0, ut, du0: shape (2, ny, nx).  Returns (L, dL)."""
    u0 = np.ascontiguousarray(u0, dtype=np.float64)
    ut = np.ascontiguousarray(ut, dtype=np.float64)
    _, ny, nx = u0.shape
    assert ut.shape == u0.shape
    d = None
    if du0 is not None:
        d = np.ascontiguousarray(du0, dtype=np.float64)
        assert d.shape == u0.shape
    t = np.array([float(taus[0]), float(taus[1] if len(taus) > 1 else taus[0])])
    out = np.zeros(2)
    arr = (OrcBC * max(1, len(bcs)))(*bcs)
    rc = lib().orc_tangent_loss(qid(q), {"SRT": 0, "TRT": 1, "MRT": 2}[kind], t, np.array(F, dtype=np.float64), nx, ny,
                                u0, ut, np.array(seed, dtype=np.float64),
                                d.ctypes.data if d is not None else None, int(nsteps), int(nthreads),
                                C.cast(arr, C.c_void_p) if len(bcs) else None, len(bcs), out)
    if rc != 0:
        raise ValueError(f"orc_tangent_loss: status {rc}")
    return float(out[0]), float(out[1])


def max_threads() -> int:
    return int(lib().orc_max_threads())
