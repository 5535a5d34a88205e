"""Convergence studies and parameter sweeps run as device batches.

The reference runs one `simulate` per (N, q, τ) point (examples/notebooks/taylor_green_vortex.ipynb
cell 3: TGV(q, τ, scale, Nx·scale, Ny·scale, u0/scale) simulated to its decay time, error from
TrackHydrodynamicErrors at the last step).  Here every point is a lattice of one DeviceBatch, so
the whole study advances with one CUDA-graph launch; errors are then reduced per lattice on the
device.
"""
from __future__ import annotations

import math
import time

import numpy as np

from .device import DeviceBatch
from .initial_conditions import AnalyticalEquilibrium
from .model import LatticeBoltzmannModel
from .problems import TGV
from .processing_methods import track_errors
from .quadratures import Quadratures


def tgv_instances(n_instances=48, sizes=(16, 32, 64, 128, 256, 512, 1024), quadratures=("D2Q9", "D2Q17"),
                  tau_range=(0.51, 2.0), seed=20240612, steps_per_n2=1 / 256, u0_times_n=0.16):
    """The study's points: (N, q) pairs round-robin over sizes x quadratures, τ uniform from a
    seeded generator, steps = max(1, round(N² · steps_per_n2)) (a fixed physical time under
    diffusive scaling), initial amplitude u0 = u0_times_n / N (the notebook's u0 / scale)."""
    rng = np.random.default_rng(seed)
    pairs = [(n, q) for n in sizes for q in quadratures]
    out = []
    for k in range(n_instances):
        n, q = pairs[k % len(pairs)]
        tau = float(rng.uniform(*tau_range))
        out.append({"N": n, "q": q, "tau": tau, "u0": u0_times_n / n, "steps": max(1, int(round(n * n * steps_per_n2)))})
    return out


def build_tgv_models(instances, storage="df64dev"):
    models = []
    for ins in instances:
        q = Quadratures[ins["q"]]
        problem = TGV(q, ins["tau"], 1, ins["N"], ins["N"], ins["u0"])
        models.append(LatticeBoltzmannModel(problem, q, collision_model=_srt(problem, q),
                                            initialization_strategy=AnalyticalEquilibrium(), storage=storage))
    return models


def _srt(problem, q):
    from .collision_models import SRT
    return SRT(q.speed_of_sound_squared * problem.lattice_viscosity() + 0.5)


def convergence_order(instances, errors, key="error_u"):
    """Least-squares slope of -log(error) against log(N), per velocity set."""
    orders = {}
    for q in sorted({ins["q"] for ins in instances}):
        xs, ys = [], []
        for ins, e in zip(instances, errors):
            v = getattr(e, key)
            if ins["q"] == q and v > 0 and math.isfinite(v):
                xs.append(math.log(ins["N"]))
                ys.append(math.log(v))
        if len(xs) >= 2:
            orders[q] = float(-np.polyfit(xs, ys, 1)[0])
    return orders


def run_tgv_study(instances=None, storage="df64dev", sequential=True, torch=None):
    """Runs the study batched (one graph) and, if `sequential`, once more one lattice after
    another, timing both with CUDA events.  Returns a dict of timings, MLUPS, errors, orders."""
    if torch is None:
        import torch
    instances = instances or tgv_instances()
    steps = np.array([ins["steps"] for ins in instances], dtype=np.int64)
    lu = float(sum(ins["N"] ** 2 * ins["steps"] for ins in instances))
    res = {"instances": len(instances), "lattice_updates": lu, "storage": storage}

    models = build_tgv_models(instances, storage)
    batch = DeviceBatch([m.lattice for m in models])
    stream = torch.cuda.Stream()
    batch.set_stream(stream.cuda_stream)
    torch.cuda.synchronize()
    # warm-up: capture the graph on a throw-away copy of the states is not needed; the first
    # call captures, so time a second call from the same initial states
    f0 = [m.f_stream for m in models]
    batch.step(steps)
    batch.synchronize()
    for m, f in zip(models, f0):
        m.lattice.upload(f)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    batch.step(steps)
    e1.record(stream)
    e1.synchronize()
    res["batched_s"] = e0.elapsed_time(e1) / 1e3
    res["batched_mlups"] = lu / res["batched_s"] / 1e6
    res["graph_kernel_launches"] = batch.last_launch_count()
    errors = [track_errors(m, m.problem, ins["steps"]) for m, ins in zip(models, instances)]
    res["orders"] = convergence_order(instances, errors)
    res["errors"] = [{"N": ins["N"], "q": ins["q"], "tau": ins["tau"], "steps": ins["steps"],
                      "error_u": e.error_u, "error_p": e.error_p} for ins, e in zip(instances, errors)]
    batch.close()

    if sequential:
        for m, f in zip(models, f0):
            m.lattice.upload(f)
        torch.cuda.synchronize()
        t0 = time.perf_counter()  # one lattice after another, each on its own stream
        for m, ins in zip(models, instances):
            m.lattice.step(ins["steps"], 0, 1.0)
            m.lattice.synchronize()
        res["sequential_s"] = time.perf_counter() - t0
        res["sequential_mlups"] = lu / res["sequential_s"] / 1e6
        res["speedup_vs_sequential"] = res["sequential_s"] / res["batched_s"]
        seq_errors = [track_errors(m, m.problem, ins["steps"]) for m, ins in zip(models, instances)]
        res["max_rel_diff_batched_vs_sequential"] = float(max(
            abs(a.error_u - b.error_u) / max(abs(b.error_u), 1e-300) for a, b in zip(errors, seq_errors)))
    for m in models:
        m.close()
    return res


# ---------------------------------------------------------------------------------------
# The TRT relaxation-time sweep of examples/notebooks/trt_magic_parameter.ipynb
# ---------------------------------------------------------------------------------------
def trt_sweep_points(taus_s, taus_a=None):
    """All (τ_s, τ_a) pairs of the notebook's `for τ_s in τ_s_range, τ_a in τ_a_range` loop."""
    taus_a = taus_s if taus_a is None else taus_a
    return [(float(ts), float(ta)) for ts in taus_s for ta in taus_a]


def julia_range(start, stop, step):
    """Julia's range(start, stop=stop, step=step) of decimal literals: the element k is the double
    nearest start + k·step taken exactly (what Julia's twice-precision ranges give for such
    literals, e.g. 0.61 rather than 0.51 + 0.1), k = 0 .. floor((stop - start) / step)."""
    from decimal import Decimal
    a, b, h = Decimal(repr(start)), Decimal(repr(stop)), Decimal(repr(step))
    n = int((b - a) // h) + 1
    return [float(a + k * h) for k in range(n)]


def build_trt_sweep_models(points, scale=1, quadrature="D2Q9", storage="f64"):
    """One model per point as `solve(problem, q, τ_s, τ_a)` of the notebook builds it:
    PoiseuilleFlow(ν, scale) with ν = (τ_s - 1/2) c_s², t_end = 100, TRT(τ_s, τ_a) with the
    problem's lattice force, TrackHydrodynamicErrors(problem, false, n_steps,
    VelocityConvergenceStoppingCriteria(1e-7, problem)), zero-velocity start.  Returns the
    models and their time ranges 0:n_steps."""
    from .collision_models import TRT
    from .initial_conditions import ZeroVelocityInitialCondition
    from .problems import PoiseuilleFlow
    from .processing_methods import TrackHydrodynamicErrors, VelocityConvergenceStoppingCriteria
    q = Quadratures[quadrature]
    models, times = [], []
    for ts, ta in points:
        problem = PoiseuilleFlow((ts - 0.5) / q.speed_of_sound_squared, scale)
        n_steps = int(round(100.0 / problem.delta_t()))
        pm = TrackHydrodynamicErrors(problem, False, n_steps, VelocityConvergenceStoppingCriteria(1e-7, problem))
        models.append(LatticeBoltzmannModel(problem, q, collision_model=TRT.fields(ts, ta, "problem"),
                                            initialization_strategy=ZeroVelocityInitialCondition(),
                                            process_method=pm, storage=storage))
        times.append(range(0, n_steps + 1))
    return models, times


def run_trt_sweep(points, scale=1, storage="f64", batched=True, sequential_points=None, torch=None, warmup=True):
    """The sweep batched (simulate_batch over all points) and, for `sequential_points` (a
    subset, or all), one simulate after another.  Both arms build their models first and time
    the time loops alone (wall clock, synchronised); with `warmup`, a few points run untimed first
    through each arm, so that the kernels' one-time loading is not timed.  Returns rows, timings
    and runs per second."""
    from .model import simulate_batch, simulate_model
    if torch is None:
        import torch
    res = {"points": len(points), "scale": scale, "storage": storage}
    rows = {}
    if warmup:
        if batched:
            wm, wt = build_trt_sweep_models(points[:8], scale, storage=storage)
            simulate_batch(wm, wt)
            for m in wm:
                m.close()
        if sequential_points:
            wm, wt = build_trt_sweep_models(sequential_points[:1], scale, storage=storage)
            simulate_model(wm[0], wt[0])
            wm[0].close()
    if batched:
        t0 = time.perf_counter()
        models, times = build_trt_sweep_models(points, scale, storage=storage)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        simulate_batch(models, times)
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        res["batched_setup_s"] = t1 - t0
        res["batched_s"] = t2 - t1
        res["batched_runs_per_s"] = len(points) / (t2 - t1)
        res["batched_steps"] = int(sum(m.processing_method.df[-1].timestep for m in models))
        for p, m in zip(points, models):
            rows[p] = m.processing_method.df[-1]
            m.close()
    if sequential_points:
        t0 = time.perf_counter()
        models, times = build_trt_sweep_models(sequential_points, scale, storage=storage)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        for m, tm in zip(models, times):
            simulate_model(m, tm)
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        res["sequential_points"] = len(sequential_points)
        res["sequential_setup_s"] = t1 - t0
        res["sequential_s"] = t2 - t1
        res["sequential_runs_per_s"] = len(sequential_points) / (t2 - t1)
        diffs = []
        for p, m in zip(sequential_points, models):
            r = m.processing_method.df[-1]
            if p in rows:
                b = rows[p]
                diffs.append(max(abs(x - y) / max(abs(y), 1e-300) for x, y in zip(b, r)
                                 if math.isfinite(x) and math.isfinite(y)))
            m.close()
        if diffs:
            res["max_rel_diff_batched_vs_sequential"] = float(max(diffs))
        if batched:
            res["speedup_vs_sequential"] = res["batched_runs_per_s"] / res["sequential_runs_per_s"]
    res["rows"] = rows
    return res


# The columns of the notebook's `results` (trt_magic_parameter.ipynb cell 2, the NamedTuple that
# `push!(s, (τ_s = …, τ_a = …, quadrature = q, error_u = …, …))` builds, shown as a 902500×7
# DataFrame in cell 3).
SWEEP_COLUMNS = ("τ_s", "τ_a", "quadrature", "error_u", "error_p", "error_σ_xx", "error_σ_xy")


def trt_sweep_table(rows, quadrature="D2Q9"):
    """The sweep's `results` as a column table: `rows` maps (τ_s, τ_a) to the last TrackRow of
    that run (run_trt_sweep's "rows"); the order is that of `rows` (the notebook's loop order
    when the points came from trt_sweep_points).  Returns {column: numpy array}."""
    keys = list(rows)
    table = {"τ_s": np.array([k[0] for k in keys], dtype=np.float64),
             "τ_a": np.array([k[1] for k in keys], dtype=np.float64),
             "quadrature": np.array([quadrature] * len(keys), dtype="U8")}
    for col in SWEEP_COLUMNS[3:]:
        table[col] = np.array([getattr(rows[k], col) for k in keys], dtype=np.float64)
    return table


def save_sweep_table(path, table):
    """Writes the table as an uncompressed .npz (one array per column, the column names as the
    array names), the stand-in for the notebook's `@save "trt_magic_parameter_001.jld2" results`:
    JLD2 is an HDF5 file that needs Julia or an HDF5 library, and neither is part of this
    package's dependencies.  Julia reads the file with NPZ.jl's `npzread`."""
    missing = [c for c in SWEEP_COLUMNS if c not in table]
    if missing:
        raise ValueError(f"sweep table lacks the columns {missing}")
    n = {len(table[c]) for c in SWEEP_COLUMNS}
    if len(n) != 1:
        raise ValueError("sweep table columns differ in length")
    with open(path, "wb") as fh:
        np.savez(fh, **{c: np.asarray(table[c]) for c in SWEEP_COLUMNS})


def load_sweep_table(path):
    """The table save_sweep_table wrote (`@load "trt_magic_parameter_001.jld2"`, cell 5)."""
    with np.load(path, allow_pickle=False) as z:
        return {c: z[c].copy() for c in SWEEP_COLUMNS}


def sweep_error_grid(table, column="error_u"):
    """The notebook's contour input (cells 6-7): τ_ss and τ_as (the unique values in order of
    first appearance, as `unique` gives them) and grid[a, s] = the column's value at
    (τ_ss[s], τ_as[a]), NaN where the sweep has no such point; `contour(τ_ss, τ_as, f)`
    evaluates f(τ_s, τ_a) over x = τ_ss, y = τ_as, so rows follow τ_a."""
    ts = table["τ_s"]
    ta = table["τ_a"]
    s_vals = list(dict.fromkeys(ts.tolist()))
    a_vals = list(dict.fromkeys(ta.tolist()))
    s_idx = {v: k for k, v in enumerate(s_vals)}
    a_idx = {v: k for k, v in enumerate(a_vals)}
    grid = np.full((len(a_vals), len(s_vals)), np.nan)
    for s, a, e in zip(ts.tolist(), ta.tolist(), np.asarray(table[column]).tolist()):
        grid[a_idx[a], s_idx[s]] = e
    return np.array(s_vals), np.array(a_vals), grid


# ---------------------------------------------------------------------------------------
# The shear-wave convergence analysis of examples/notebooks/shear_wave.ipynb
# ---------------------------------------------------------------------------------------
def build_shear_wave_study_models(quadratures, tau=0.8, scales=(1, 2, 4, 8), storage="f64"):
    """The runs of shear_wave_convergence_analysis(q, AnalyticalEquilibrium(), τ; scales)
    (examples/notebooks/notebook_examples.jl:34-69), which shear_wave.ipynb calls for every
    quadrature: per quadrature and scale, DecayingShearFlow(ν, scale, static = true) with
    ν = τ / (2 speed_of_sound_squared) as written there, n_steps = round(t_end / Δt) for t_end = 1,
    TrackHydrodynamicErrors(problem, false, n_steps, NoStoppingCriteria()), the default SRT
    collision and the analytical-equilibrium start.  The static flow carries a time-dependent
    force (decaying_shear_flow.jl:132-147).  Returns the models, their time ranges 0:n_steps
    and the (quadrature, scale) of each."""
    from .collision_models import SRT
    from .problems import DecayingShearFlow
    from .processing_methods import NoStoppingCriteria, TrackHydrodynamicErrors
    models, times, keys = [], [], []
    for qname in quadratures:
        q = Quadratures[qname]
        nu = tau / (2.0 * q.speed_of_sound_squared)
        for scale in scales:
            problem = DecayingShearFlow(nu, scale, static=True)
            n_steps = int(round(1.0 / problem.delta_t()))
            pm = TrackHydrodynamicErrors(problem, False, n_steps, NoStoppingCriteria())
            models.append(LatticeBoltzmannModel(problem, q, collision_model=SRT,
                                                initialization_strategy=AnalyticalEquilibrium(), process_method=pm,
                                                storage=storage))
            times.append(range(0, n_steps + 1))
            keys.append((qname, scale))
    return models, times, keys


def run_shear_wave_study(quadratures=("D2Q4", "D2Q5", "D2Q9", "D2Q13", "D2Q17", "D2Q21", "D2Q37"), tau=0.8,
                         scales=(1, 2, 4, 8), storage="f64", sequential=True, torch=None, warmup=True):
    """The study batched (simulate_batch: every run in one batch, the time-dependent force of each
    member evaluated at its own step times) and, if `sequential`, once more one simulate after
    another.  Both arms build their models first and time the time loops alone; with `warmup`,
    each arm first runs once untimed on models of its own, so that the kernels' one-time loading
    is not timed.  Returns the final rows, timings, and the convergence order of error_u per
    quadrature."""
    from .model import simulate_batch, simulate_model
    if torch is None:
        import torch
    res = {"runs": len(quadratures) * len(scales), "storage": storage, "tau": tau, "scales": list(scales)}
    if warmup:
        wm, wt, _ = build_shear_wave_study_models(quadratures, tau, scales, storage)
        simulate_batch(wm, wt)
        for m in wm:
            m.close()
        if sequential:
            wm, wt, _ = build_shear_wave_study_models(quadratures, tau, scales, storage)
            for m, tm in zip(wm, wt):
                simulate_model(m, tm)
                m.close()
    models, times, keys = build_shear_wave_study_models(quadratures, tau, scales, storage)
    res["lattice_updates"] = float(sum(m.lattice.nx * m.lattice.ny * (tm.stop - 1) for m, tm in zip(models, times)))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    simulate_batch(models, times)
    torch.cuda.synchronize()
    res["batched_s"] = time.perf_counter() - t0
    rows = {k: m.processing_method.df[-1] for k, m in zip(keys, models)}
    for m in models:
        m.close()
    if sequential:
        models, times, _ = build_shear_wave_study_models(quadratures, tau, scales, storage)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for m, tm in zip(models, times):
            simulate_model(m, tm)
        torch.cuda.synchronize()
        res["sequential_s"] = time.perf_counter() - t0
        res["speedup_vs_sequential"] = res["sequential_s"] / res["batched_s"]
        diffs = []
        for k, m in zip(keys, models):
            a, b = rows[k], m.processing_method.df[-1]
            diffs.append(max(abs(x - y) / max(abs(y), 1e-300) for x, y in zip(a, b)
                             if math.isfinite(x) and math.isfinite(y)))
            m.close()
        res["max_rel_diff_batched_vs_sequential"] = float(max(diffs))
    orders = {}
    for qname in quadratures:
        xs = [math.log(8 * s) for s in scales]
        ys = [rows[(qname, s)].error_u for s in scales]
        if all(y > 0 and math.isfinite(y) for y in ys):
            orders[qname] = float(-np.polyfit(xs, [math.log(y) for y in ys], 1)[0])
    res["orders"] = orders
    res["rows"] = rows
    return res
