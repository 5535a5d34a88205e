"""Benchmark of the GB300 collide-stream path on the reference's headline workload:
D2Q9 TRT (magic Λ = 1/4) Poiseuille channel, 4096 x 4096 nodes, bounce-back walls North and
South, periodic in x, constant body force Fx = 1e-6 (lattice units), τ_s drawn uniformly
from [0.55, 1.5] with a fixed seed, ρ = 1, u = 0 start.

One benchmark step is one lattice-Boltzmann time step (collide -> stream -> bounce-back) of
the whole 4096^2 lattice; the default run times 2000 steps, the configuration's run length.
`value` is MLUPS (million lattice updates per second) with the populations resident in HBM
(FP64 storage, FP64 arithmetic); `e2e` is the same metric through the C ABI with the host
arrays copied in and out inside the timed region.  Extra keys report the FP32-deviation
storage and the CPU baseline (the oracle port on the host cores).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NX = NY = 4096
Q = 9
SEED = 20240611
METRIC = "D2Q9 TRT 4096² MLUPS & %HBM peak: FP64 vs FP32-dev, batched, adjoint"
BYTES_PER_LU = {"f64": 2 * Q * 8, "df64dev": 2 * Q * 8, "f32dev": 2 * Q * 4, "f16dev": 2 * Q * 2, "f32sr": 2 * Q * 4,
                "f64dd": 2 * Q * 8}
ACCURACY_STEPS = 2000  # the configuration's run length, over which each storage's error is measured


def tau_from_seed():
    rng = np.random.default_rng(SEED)
    return float(rng.uniform(0.55, 1.5))


def peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return None


def profiled_traffic():
    """DRAM bytes per launch of the fused step kernel from the committed ncu summary."""
    try:
        return json.load(open(os.path.join(ROOT, "profiles", "traffic.json")))
    except Exception:
        return {}


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        try:
            for line in open(self.path):
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    mx = float(parts[2])
                except ValueError:
                    continue
                names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
                for name, v in zip(names, parts[5:9]):
                    if v.lower() == "active":
                        reasons.add(name)
        except Exception:
            pass
        finally:
            try:
                os.unlink(self.path)
            except Exception:
                pass
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def build_model(lbm, storage, tau_s, n=None):
    q = lbm.D2Q9()
    nu = (tau_s - 0.5) / q.speed_of_sound_squared
    u_max = 0.05
    nx = ny = n or NX
    problem = lbm.PoiseuilleFlow.fields(1.0, u_max, nu, nx, ny, 1.0, (1.0, 1.0), 1.0)
    problem.G = 1e-6 / (u_max * problem.delta_t() * problem.viscosity())  # lattice force 1e-6
    cm = lbm.TRT.fields(tau_s, 0.5 + 0.25 / (tau_s - 0.5), "problem")
    f0 = lbm.initialize(lbm.ZeroVelocityInitialCondition(), q, problem)
    model = lbm.LatticeBoltzmannModel(problem, q, collision_model=cm, storage=storage, f0=f0)
    return problem, model, f0


def time_device(torch, model, steps, warmup, dt):
    """K steps timed with CUDA events on the stream the kernels run on."""
    stream = torch.cuda.Stream()
    model.lattice.set_stream(stream.cuda_stream)
    with torch.cuda.stream(stream):
        model.lattice.step(warmup, 0, dt)
        torch.cuda.synchronize()
        start = torch.cuda.Event(enable_timing=True)
        end = torch.cuda.Event(enable_timing=True)
        start.record(stream)
        model.lattice.step(steps, warmup, dt)
        end.record(stream)
        end.synchronize()
        torch.cuda.synchronize()
    launches = model.lattice.last_launch_count()
    return start.elapsed_time(end) / 1e3, launches


def time_e2e(torch, lbm, problem, model, f0, steps, dt):
    """Upload from pinned host memory, K steps, download to pinned host memory."""
    stream = torch.cuda.Stream()
    model.lattice.set_stream(stream.cuda_stream)
    host_in = torch.from_numpy(f0).pin_memory()
    host_out = torch.empty_like(host_in).pin_memory()
    torch.cuda.synchronize()
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        start.record(stream)
        model.lattice.upload(host_in)
        model.lattice.step(steps, 0, dt)
        model.lattice.download(host_out)
        end.record(stream)
        end.synchronize()
    return start.elapsed_time(end) / 1e3, host_in.numel() * 8, host_out.numel() * 8


def oracle_channel(O, tau_s, nx=NX, ny=NY):
    """The benchmark channel as oracle inputs: problem, TRT collision with the force, the
    bounce-back walls and the zero-velocity start (f = w)."""
    nu = (tau_s - 0.5) / 3.0
    p = O.poiseuille_struct(1.0, 0.05, nu, nx, ny, 1.0, (1.0, 1.0), 1.0)
    sc = O.problem_scalars(p)
    p.G = 1e-6 / (0.05 * sc["delta_t"] * sc["viscosity"])
    cm = O.collision("TRT", [tau_s, 0.5 + 0.25 / (tau_s - 0.5)], force=True)
    bcs = [O.bc("bounce_back", "north", (1, nx), (1, ny)), O.bc("bounce_back", "south", (1, nx), (1, ny))]
    return p, cm, bcs, O.initialize(O.INIT_ZERO_VELOCITY, "D2Q9", p), sc["delta_t"]


def cpu_rate(tau_s, threads, budget_s):
    """The oracle port (collide -> stream -> bounce-back, OpenMP over x) on `threads` host
    threads, on a bounded sample of the workload: whole 4096^2 time steps, as many as fit the
    budget after one warm-up step."""
    from oracle import oracle as O
    p, cm, bcs, f, dt = oracle_channel(O, tau_s)
    t0 = time.perf_counter()
    f = O.run("D2Q9", p, cm, bcs, f, 0, 0, dt=dt, nthreads=threads)
    one = time.perf_counter() - t0
    n = max(1, min(50, int(budget_s / max(one, 1e-3))))
    t0 = time.perf_counter()
    O.run("D2Q9", p, cm, bcs, f, 1, n, dt=dt, nthreads=threads)
    el = time.perf_counter() - t0
    return {"value": NX * NY * n / el / 1e6, "unit": "MLUPS", "cores": threads, "kind": "port",
            "sample": f"{n} time steps of the full {NX}x{NY} lattice (after 1 warm-up step), "
                      f"{threads} OpenMP thread{'s' if threads > 1 else ''}, C++ restatement of the reference loop"}


def cpu_model():
    """The host CPU's model name (lscpu), else what /proc/cpuinfo or the platform gives."""
    import platform
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name"):
                return f"{line.split(':', 1)[1].strip()} ({platform.machine()})"
    except Exception:
        pass
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu part")):
                return f"{line.split(':', 1)[1].strip()} ({platform.machine()})"
    except Exception:
        pass
    return platform.processor() or platform.machine()


def cpu_baseline(tau_s, budget_s=12.0):
    """The oracle port on all host cores (the reported baseline) and on one core (the reference
    itself is single-threaded: src/ has no threading), each on a bounded sample."""
    from oracle import oracle as O
    threads = O.max_threads()
    res = cpu_rate(tau_s, threads, budget_s)
    res["single_thread"] = cpu_rate(tau_s, 1, budget_s) if threads > 1 else dict(res)
    res["cpu"] = cpu_model()
    return res


def bench_tgv64(torch, lbm, storage="f64"):
    """Taylor-Green vortex 64 x 64, D2Q9 SRT τ = 0.8, equilibrium + off-equilibrium start, 1000
    steps, TrackHydrodynamicErrors at step 1000 (the CPU-runnable configuration)."""
    q = lbm.D2Q9()
    problem = lbm.TaylorGreenVortex(0.1, 1, 64, 64, static=False)
    pm = lbm.TrackHydrodynamicErrors(problem, False, 1000)
    t0 = time.perf_counter()
    m = lbm.LatticeBoltzmannModel(problem, q, collision_model=lbm.SRT, process_method=pm, storage=storage,
                                  initialization_strategy=lbm.AnalyticalEquilibriumAndOffEquilibrium())
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    lbm.simulate(m, time=range(0, 1000))
    t2 = time.perf_counter()
    row = pm.df[-1]
    m.close()
    return {"workload": "D2Q9 SRT Taylor-Green vortex 64x64, tau=0.8, 1000 steps, FP64", "storage": storage,
            "simulate_s": t2 - t1, "setup_s": t1 - t0, "mlups": 64 * 64 * 1000 / (t2 - t1) / 1e6,
            "error_u": row.error_u, "error_p": row.error_p, "error_sigma_xx": row.error_σ_xx,
            "error_sigma_xy": row.error_σ_xy}


def bench_mrt_d2q37(torch, lbm, steps=500, n=2048):
    """Regularised MRT D2Q37 shear wave n x n, τ = 0.6, u_x = 0.01 sin(2π y / n), 500 steps:
    MLUPS, HBM fraction and the velocity / stress errors against the analytic decay."""
    q = lbm.D2Q37()
    tau = 0.6
    problem = lbm.ShearWave(n, n, (tau - 0.5) / q.speed_of_sound_squared, 0.01)
    f0 = lbm.initialize(lbm.AnalyticalEquilibrium(), q, problem)
    pk = peaks()
    peak = pk["hbm_gbs"] if pk else 6800.0
    out = {"workload": f"D2Q37 regularised MRT shear wave {n}x{n}, tau=0.6, {steps} steps"}
    for storage, esize in (("f64", 8), ("df64dev", 8), ("f32dev", 4), ("f64dd", 8), ("f32sr", 4)):
        m = lbm.LatticeBoltzmannModel(problem, q, collision_model=lbm.MRT(q, tau), storage=storage, f0=f0)
        st = steps if storage not in ("f64", "f64dd") else max(20, steps // (10 if storage == "f64" else 4))
        sec, _ = time_device(torch, m, st, 3, 1.0)
        row = lbm.track_errors(m, problem, st + 3)
        m.close()
        mlups = n * n * st / sec / 1e6
        out[storage] = {"mlups": mlups, "steps_timed": st, "hbm_frac": 2 * 37 * esize * mlups * 1e6 / 1e9 / peak,
                        "error_u": row.error_u, "error_sigma_xy": row.error_σ_xy}
    return out


def bench_batched(torch, lbm):
    """The convergence study in FP64 (the study's own precision) and in float-float storage."""
    out = {"workload": ("48 Taylor-Green lattices N in {16..1024}^2 x {D2Q9, D2Q17}, tau ~ U[0.51, 2.0] (seeded), "
                        "steps = N^2/256, one CUDA graph vs one lattice after another; FP64 and float-float storage")}
    for storage in ("f64", "df64dev"):
        res = lbm.run_tgv_study(storage=storage, torch=torch)
        res.pop("errors", None)
        out[storage] = res
    return out


def bench_trt_sweep(torch, lbm, every=40):
    """The TRT relaxation-time sweep of trt_magic_parameter.ipynb (cell 2's grid τ_s, τ_a in
    0.51:0.1:10.0, 9025 Poiseuille runs of PoiseuilleFlow(ν, 1), TRT with force, velocity
    convergence stop at 1e-7, t_end = 100): all runs batched, and every `every`-th run one after
    another for the sequential rate; rows of the common runs must agree bitwise."""
    taus = lbm.julia_range(0.51, 10.0, 0.1)
    pts = lbm.trt_sweep_points(taus)
    res = lbm.run_trt_sweep(pts, scale=1, sequential_points=pts[::every], torch=torch)
    rows = res.pop("rows")
    res["workload"] = ("TRT (tau_s, tau_a) sweep of trt_magic_parameter.ipynb: 95 x 95 = 9025 D2Q9 Poiseuille "
                       "runs (3 x 5 nodes, force, bounce-back, velocity-convergence stop), FP64; sequential "
                       f"rate from every {every}th run")
    best = min(rows.items(), key=lambda kv: kv[1].error_u if math.isfinite(kv[1].error_u) else math.inf)
    res["best_point"] = {"tau_s": best[0][0], "tau_a": best[0][1], "error_u": best[1].error_u}
    return res


def bench_shear_wave_study(torch, lbm):
    """The shear-wave convergence analysis of shear_wave.ipynb for every quadrature
    (notebook_examples.jl:34-69: DecayingShearFlow(ν, scale, static = true), its time-dependent
    force, SRT, t_end = 1, scales 1, 2, 4, 8): 28 runs in one batch vs one simulate after another."""
    res = lbm.run_shear_wave_study(torch=torch)
    rows = res.pop("rows")
    res["error_u"] = {f"{q}-{s}": r.error_u for (q, s), r in rows.items()}
    res["workload"] = ("shear-wave convergence analysis of shear_wave.ipynb: D2Q4..D2Q37 x scales 1, 2, 4, 8, "
                       "DecayingShearFlow(static = true) with its time-dependent force, SRT tau = 0.8, t_end = 1, FP64")
    return res


def bench_all_sets(torch, lbm, n=2048, steps=40):
    """Every velocity set, TRT, periodic n x n, zero-velocity start plus a constant force: the
    fused step's MLUPS and fraction of the measured HBM bandwidth per storage (2 Q sizeof(T)
    bytes per update)."""
    pk = peaks()
    peak = pk["hbm_gbs"] if pk else 6800.0
    out = {"workload": f"TRT periodic {n}x{n}, Fx = 1e-6, {steps} steps per storage and velocity set"}
    for qn in ("D2Q4", "D2Q5", "D2Q9", "D2Q13", "D2Q17", "D2Q21", "D2Q37"):
        q = lbm.Quadratures[qn]
        row = {}
        for storage, esize in (("f64", 8), ("df64dev", 8), ("f32dev", 4), ("f16dev", 2)):
            lat = lbm.DeviceLattice(q, n, n, lbm.TRT.fields(0.8, 1.1), (), force=("constant", (1e-6, 0.0)),
                                    storage=storage)
            lat.initialize_fields()
            m = type("M", (), {"lattice": lat})()
            st = steps if storage != "f64" else max(4, steps // 4)
            sec, _ = time_device(torch, m, st, 3, 0.0)
            lat.close()
            mlups = n * n * st / sec / 1e6
            row[storage] = {"mlups": mlups, "hbm_frac": 2 * q.Q * esize * mlups * 1e6 / 1e9 / peak}
        out[qn] = row
    return out


def bench_init(torch, lbm, n=2048):
    """Model construction with the Taylor-Green equilibrium + off-equilibrium initial condition:
    the state built on the device from the macroscopic planes, against the host build of all Q
    planes and their upload (the reference's initialize loop, vectorised)."""
    q = lbm.D2Q9()
    problem = lbm.TaylorGreenVortex(0.1, 1, n, n, static=False)
    st = lbm.AnalyticalEquilibriumAndOffEquilibrium()
    out = {"workload": f"LatticeBoltzmannModel(TaylorGreenVortex {n}x{n}, D2Q9, equilibrium + off-equilibrium)"}
    f = {}
    for name, dev in (("device_s", True), ("host_s", False)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        m = lbm.LatticeBoltzmannModel(problem, q, initialization_strategy=st, device_init=dev)
        torch.cuda.synchronize()
        out[name] = time.perf_counter() - t0
        f[name] = m.f_stream
        m.close()
    out["speedup"] = out["host_s"] / out["device_s"]
    out["max_abs_diff"] = float(np.max(np.abs(f["device_s"] - f["host_s"])))
    return out


def bench_adjoint(torch, lbm, n=512, steps=4000):
    q = lbm.D2Q9()
    tau_s = 0.8
    out = {"workload": f"adjoint of D2Q9 TRT {n}x{n} periodic, {steps} steps, loss = |u_T - u*|^2, "
                       "divergence-free Fourier start (k <= 8, amplitude 0.01), binomial checkpointing"}
    u0 = lbm.divergence_free_field(n, n, 8, 0.01, seed=11)
    ut = lbm.divergence_free_field(n, n, 8, 0.01, seed=12)
    for st in ("f32dev",):
        prob = lbm.AdjointProblem(q, n, n, lbm.TRT.fields(tau_s, lbm.trt_magic(tau_s)), force=(1e-6, 0.0),
                                  nsteps=steps, storage=st)
        prob.run(u0, ut, want_grad_u0=False)  # captures the graph
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res = prob.run(u0, ut)
        t1 = time.perf_counter()
        info = prob.info()
        prob.close()
        out[st] = {"seconds": t1 - t0, "forward_equivalent_mlups": n * n * steps / (t1 - t0) / 1e6,
                   "loss": res["loss"], "dL_dtau_s_total": lbm.magic_total_derivative(res, tau_s),
                   "dL_dF": [float(x) for x in res["dF"]], "checkpoint_slots": info["slots"],
                   "forward_steps": info["forward_steps"], "device_bytes": info["device_bytes"],
                   "state_bytes": n * n * 9 * 4}
    # a memory budget: 8 slots instead of the default (every step recomputed at most r times,
    # C(8 + r, 8) >= T), the walled channel (bounce-back North / South), and the regularised MRT
    trt = lbm.TRT.fields(tau_s, lbm.trt_magic(tau_s))
    walls = [lbm.BounceBack(lbm.North(), (1, n), (1, n)), lbm.BounceBack(lbm.South(), (1, n), (1, n))]
    for label, cm, kw in (("f32dev_8_slots", trt, {"slots": 8}),
                          ("f32dev_channel_walls", trt, {"boundary_conditions": walls}),
                          ("f32dev_mrt", lbm.MRT(q, tau_s), {})):
        prob = lbm.AdjointProblem(q, n, n, cm, force=(1e-6, 0.0), nsteps=steps, storage="f32dev", **kw)
        prob.run(u0, ut, want_grad_u0=False)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res = prob.run(u0, ut)
        t1 = time.perf_counter()
        info = prob.info()
        prob.close()
        out[label] = {"seconds": t1 - t0, "loss": res["loss"], "checkpoint_slots": info["slots"],
                      "forward_steps": info["forward_steps"], "device_bytes": info["device_bytes"]}
    return out


def finite(obj):
    """The JSON line carries no NaN / Infinity tokens (they are not JSON): such values become null."""
    if isinstance(obj, float):
        return obj if math.isfinite(obj) else None
    if isinstance(obj, dict):
        return {k: finite(v) for k, v in obj.items()}
    if isinstance(obj, (list, tuple)):
        return [finite(v) for v in obj]
    return obj


def max_over_ranks(seconds, world, device):
    """The slowest rank's time: every rank runs its own replica of the lattice (the path has no
    exchange step at one lattice per GPU), and the job ends when the last replica does."""
    if world <= 1:
        return float(seconds)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_mlups(updates_per_rank, seconds, world):
    """Whole-job MLUPS: the lattice updates of all replicas over the slowest rank's time."""
    return updates_per_rank * world / seconds / 1e6


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def run_reference(args):
    """The reference arm: the oracle port of the reference loop on all host threads (the
    reference is Julia, absent on the box), timed over exactly `--steps` steps after `--warmup`
    untimed ones.  A step is one time step of a 4096-wide channel: the full 4096 rows when the
    run fits a few minutes, else a strip of fewer rows (walls North / South, same τ and force),
    so that steps x ms_per_step is the timed region."""
    world, rank, _ = dist_setup(args)
    if rank != 0:
        return 0
    tau_s = tau_from_seed()
    from oracle import oracle as O
    O.build()
    threads = O.max_threads()
    steps, warmup = max(1, args.steps), max(0, args.warmup)
    # ~0.4 s per full step on 16 cores: full lattice up to 100 steps in all, else fewer rows
    ny = NY if steps + warmup <= 100 else max(64, (NY * 100 // (steps + warmup)) // 8 * 8)
    p, cm, bcs, f, dt = oracle_channel(O, tau_s, NX, ny)
    if warmup:
        f = O.run("D2Q9", p, cm, bcs, f, 0, warmup - 1, dt=dt, nthreads=threads)
    t0 = time.perf_counter()
    O.run("D2Q9", p, cm, bcs, f, warmup, warmup + steps - 1, dt=dt, nthreads=threads)
    el = time.perf_counter() - t0
    value = NX * ny * steps / el / 1e6
    sample = (f"{steps} time steps (after {warmup} untimed) of a {NX}x{ny} D2Q9 TRT channel"
              f"{'' if ny == NY else ' (a strip of the 4096x4096 workload, same walls, tau and force)'}, "
              f"{threads} OpenMP threads, C++ restatement of the reference loop")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "MLUPS", "n_gpus": args.gpus,
            "steps": steps, "warmup": warmup, "ms_per_step": el / steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "D2Q9 TRT Poiseuille channel, FP64, CPU oracle port (the reference is Julia, "
                                   "not runnable on the box)", "nx": NX, "ny": ny, "tau_s": tau_s,
                       "cpu": cpu_model()},
            "cpu_baseline": {"value": value, "unit": "MLUPS", "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(finite(line), allow_nan=False))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--storage", default="f64", choices=["f64", "df64dev", "f32dev", "f16dev", "f32sr", "f64dd"])
    ap.add_argument("--profile", action="store_true",
                    help="time only the device loop of the chosen storage (for profiler runs)")
    ap.add_argument("--case", default="poiseuille",
                    choices=["poiseuille", "mrt_d2q37", "trt_sweep", "adjoint", "shear_wave_study"],
                    help="with --profile: the workload run (D2Q9 TRT Poiseuille 4096^2, D2Q37 regularised MRT "
                         "shear wave 2048^2, the batched TRT sweep, the D2Q9 TRT 512^2 adjoint, or the batched "
                         "shear-wave convergence study)")
    ap.add_argument("--n", type=int, default=0,
                    help="with --profile: an n x n lattice for the Poiseuille case (default 4096) and the D2Q37 MRT case (default 2048)")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the other configurations (Taylor-Green 64^2, D2Q37 MRT, batched study, adjoint)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.warmup < 3:
        args.warmup = 3

    import torch
    world, rank, local = dist_setup(args)
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    import __graft_entry__
    lbm = __graft_entry__.load_package()
    lbm._native.lib()
    tau_s = tau_from_seed()

    if args.profile and args.case == "mrt_d2q37":
        q = lbm.D2Q37()
        n = args.n or 2048
        problem = lbm.ShearWave(n, n, (0.6 - 0.5) / q.speed_of_sound_squared, 0.01)
        f0 = lbm.initialize(lbm.AnalyticalEquilibrium(), q, problem)
        m = lbm.LatticeBoltzmannModel(problem, q, collision_model=lbm.MRT(q, 0.6), storage=args.storage, f0=f0)
        sec, launches = time_device(torch, m, args.steps, args.warmup, 1.0)
        m.close()
        print(json.dumps({"case": "mrt_d2q37", "storage": args.storage, "mlups": n * n * args.steps / sec / 1e6,
                          "launches": launches}))
        return 0
    if args.profile and args.case == "trt_sweep":  # 95 x 95 grid, every 8th point: 1129 runs
        pts = lbm.trt_sweep_points(lbm.julia_range(0.51, 10.0, 0.1))[::8]
        res = lbm.run_trt_sweep(pts, scale=1, torch=torch)
        res.pop("rows")
        print(json.dumps({"case": "trt_sweep", **res}))
        return 0
    if args.profile and args.case == "shear_wave_study":  # the 28 runs batched, once
        models, times, _ = lbm.build_shear_wave_study_models(("D2Q4", "D2Q5", "D2Q9", "D2Q13", "D2Q17", "D2Q21",
                                                              "D2Q37"))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        lbm.simulate_batch(models, times)
        torch.cuda.synchronize()
        print(json.dumps({"case": "shear_wave_study", "seconds": time.perf_counter() - t0}))
        for m in models:
            m.close()
        return 0
    if args.profile and args.n:  # a smaller channel of the same kind, for profiler captures
        problem, model, _ = build_model(lbm, args.storage, tau_s, args.n)
        sec, launches = time_device(torch, model, args.steps, args.warmup, problem.delta_t())
        model.close()
        print(json.dumps({"case": "poiseuille", "n": args.n, "storage": args.storage,
                          "mlups": args.n * args.n * args.steps / sec / 1e6, "launches": launches}))
        return 0
    if args.profile and args.case == "adjoint":
        print(json.dumps({"case": "adjoint", **bench_adjoint(torch, lbm, steps=args.steps)}))
        return 0

    problem, model, f0 = build_model(lbm, args.storage, tau_s)
    dt = problem.delta_t()
    with ClockSampler(local) as clk:
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        seconds, launches = time_device(torch, model, args.steps, args.warmup, dt)
    clocks = clk.summary()
    # velocity profile of the timed run (the flow is x-invariant: one column), the yardstick of
    # the other storages' error
    ux_ref = model.lattice.macroscopic()[1][:, 0].copy() if not args.profile else None
    seconds = max_over_ranks(seconds, world, "cuda")
    mlups = job_mlups(NX * NY * args.steps, seconds, world)
    per_launch = seconds / max(1, args.steps)
    bytes_lu = BYTES_PER_LU[args.storage]
    pk = peaks()
    peak_gbs = pk["hbm_gbs"] if pk else 6800.0
    achieved_gbs = bytes_lu * NX * NY / per_launch / 1e9
    traffic = profiled_traffic().get(f"step_{args.storage}")

    e2e = None
    if not args.profile:
        # one untimed sequence (the first transfers from freshly pinned buffers took twice as long
        # as later ones), then three complete timed sequences, the median reported
        time_e2e(torch, lbm, problem, model, f0, args.steps, dt)
        runs = [time_e2e(torch, lbm, problem, model, f0, args.steps, dt) for _ in range(3)]
        e2e_runs = [max_over_ranks(r[0], world, "cuda") for r in runs]
        e2e_s, h2d, d2h = sorted(e2e_runs)[1], runs[0][1], runs[0][2]
        # the drop-in call sequence of simulate(model, 0:K): the populations uploaded from pinned host
        # memory once before the K steps and downloaded once after them (the state stays resident
        # in between, as the reference keeps it in f_stream); bytes per step are those totals / K
        e2e = {"value": job_mlups(NX * NY * args.steps, e2e_s, world), "unit": "MLUPS",
               "h2d_bytes_per_step": h2d / args.steps, "d2h_bytes_per_step": d2h / args.steps,
               "h2d_bytes_per_call": h2d, "d2h_bytes_per_call": d2h,
               "copies": "one upload before and one download after the K-step lbm_step call",
               "runs_s": e2e_runs, "reported": "median of three complete sequences after one untimed one"}
    model.close()

    extra = {}
    if args.storage == "f64" and rank == 0 and not args.profile:
        # accuracy over the configuration's 2000 steps (untimed): every storage's velocity column
        # against the FP64 run's
        ux_acc = {}
        for st in ("f64", "df64dev", "f32dev", "f16dev", "f32sr", "f64dd"):
            _, mx, _ = build_model(lbm, st, tau_s)
            mx.lattice.step(ACCURACY_STEPS, 0, dt)
            ux_acc[st] = mx.lattice.macroscopic()[1]
            mx.close()
        ref_acc = ux_acc["f64"][:, 0]
        for st in ("df64dev", "f32dev", "f16dev", "f32sr", "f64dd"):
            _, mx, _ = build_model(lbm, st, tau_s)
            sx, _ = time_device(torch, mx, args.steps, args.warmup, dt)
            ux = mx.lattice.macroscopic()[1][:, 0]
            mx.close()
            extra[st] = {"value": NX * NY * args.steps / sx / 1e6, "unit": "MLUPS", "speedup_vs_f64": seconds / sx,
                         "roofline_frac": BYTES_PER_LU[st] * NX * NY / (sx / args.steps) / 1e9 / peak_gbs,
                         "velocity_error_vs_f64": float(np.max(np.abs(ux - ux_ref)) / np.max(np.abs(ux_ref))),
                         "error_after_steps": args.warmup + args.steps,
                         f"velocity_error_vs_f64_after_{ACCURACY_STEPS}_steps":
                             float(np.max(np.abs(ux_acc[st] - ref_acc[:, None])) / np.max(np.abs(ref_acc))),
                         "error_measure": "max over the lattice of |ux - ux_f64| / max |ux_f64|"}
        extra["f32sr"]["arithmetic"] = ("FP32 deviation storage, float-float arithmetic, collision outputs stored "
                                        "with stochastic rounding")
        extra["f64dd"]["arithmetic"] = ("FP64 storage (the f64 bytes and values), float-float arithmetic on g = f - w; "
                                        "the FP64 pipe forms g on load and w + g on store")
        extra["f64dd"]["dtype"] = "f64-storage, float-float arithmetic"
    if rank == 0 and not args.profile and not args.no_extras and args.storage == "f64":
        extra["configs"] = {"tgv64": bench_tgv64(torch, lbm), "mrt_d2q37": bench_mrt_d2q37(torch, lbm),
                            "batched": bench_batched(torch, lbm), "trt_sweep": bench_trt_sweep(torch, lbm),
                            "shear_wave_study": bench_shear_wave_study(torch, lbm),
                            "init": bench_init(torch, lbm), "all_sets": bench_all_sets(torch, lbm),
                            "adjoint": bench_adjoint(torch, lbm)}
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline and not args.profile:
        cpu = cpu_baseline(tau_s)
    if rank == 0:
        line = {"metric": METRIC, "value": mlups, "unit": "MLUPS", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": seconds / args.steps * 1e3, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": args.storage, "data": "synthetic",
                "config": {"workload": "D2Q9 TRT Poiseuille channel 4096x4096, bounce-back N/S, Fx=1e-6, "
                                       "u=0 start (one step = one time step of the whole lattice)",
                           "nx": NX, "ny": NY, "tau_s": tau_s, "tau_a": 0.5 + 0.25 / (tau_s - 0.5),
                           "storage": args.storage, "parallelism": f"replicas{world}",
                           "l2": "inputs larger than L2 (two population arrays of "
                                 f"{NX * NY * Q * bytes_lu // (2 * Q) / 1e9:.2f} GB)"},
                "roofline": {"bound": "hbm", "achieved": achieved_gbs, "peak": peak_gbs, "unit": "GB/s",
                             "frac": achieved_gbs / peak_gbs, "traffic": traffic,
                             "peak_source": "MEASURED_PEAKS.json hbm_gbs" if pk else "fallback 6.8 TB/s",
                             "bytes_per_lu": bytes_lu, "kernel": "step_kernel<D2Q9,TRT,fused>"},
                "e2e": e2e, "gpu_launches": launches, "clocks": clocks, "cpu_baseline": cpu}
        fp64_inst = profiled_traffic().get("step_f64_fp64_thread_inst_per_lu")
        if args.storage == "f64" and fp64_inst and clocks and clocks.get("sm_mhz"):
            # the FP64 step's own roof: GB300 issues 2 FP64 thread instructions per SM per clock
            sms = torch.cuda.get_device_properties(local if world > 1 else 0).multi_processor_count
            peak = sms * 2 * clocks["sm_mhz"] * 1e6 / 1e9
            ach = fp64_inst * mlups * 1e6 / 1e9
            line["compute_roofline"] = {"bound": "fp64 pipe", "achieved": ach, "peak": peak,
                                        "unit": "G FP64 thread-instructions/s", "frac": ach / peak,
                                        "instructions_per_lu": fp64_inst,
                                        "peak_source": f"{sms} SMs x 2 FP64 instructions per clock (rate measured with ncu) "
                                                       "x median SM clock of the timed region"}
        line.update(extra)
        print(json.dumps(finite(line), allow_nan=False))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
