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
