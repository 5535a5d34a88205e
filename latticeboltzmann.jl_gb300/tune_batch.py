"""Measures, on the GPU, when a batch member is faster block-resident than on the graph path, and
writes the table DeviceBatch reads (batch_schedule.json beside this file).

For every storage (f64, df64dev, f32dev) and velocity set, batches of M identical periodic TRT
lattices with a constant force are stepped K steps (the second call of each configuration is
timed with CUDA events, so graph capture is not counted), for member sizes from 24 to 4096 nodes:
  - on the graph path (schedule None), and
  - block-resident with 16, 32 and 64 nodes per CTA, each node's collision on 1, 2 or 4 warps
    (splits exist for SRT / TRT with FP64 or float-float storage from D2Q9 up).
A velocity set's row is the largest member size up to which the best resident configuration beats
the graph path at every measured size, with the configuration whose time relative to the graph
path, summed over those sizes, is least.  Both paths give the same bits, so the table changes
speed only.

  python -m latticeboltzmann_gb300.tune_batch   (or: python latticeboltzmann.jl_gb300/tune_batch.py)
"""
from __future__ import annotations

import importlib.util
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
SHAPES = ((8, 3), (16, 3), (32, 3), (64, 3), (16, 16), (32, 32), (64, 64))
PER_BLOCK = (16, 32, 64)
SPLITS = (1, 2, 4)
STORAGES = ("f64", "df64dev", "f32dev")
ELEM = {"f64": 8, "df64dev": 8, "f32dev": 4}


def _package():
    if __package__:
        import importlib
        return importlib.import_module(__package__)
    name = "latticeboltzmann_gb300"
    if name in sys.modules:
        return sys.modules[name]
    spec = importlib.util.spec_from_file_location(name, os.path.join(HERE, "__init__.py"),
                                                  submodule_search_locations=[HERE])
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


def resident_fits(Q, n, per, elem):
    """The library's rule (resident_cluster in lbm_api.cu): cluster of ceil(n / per) CTAs rounded up
    to a power of two, at most 8, and both buffers of a CTA's share within 200 KB."""
    c = 1
    while c < 8 and c * per < n:
        c *= 2
    chunk = -(-n // c)
    return 2 * Q * chunk * elem <= 200 * 1024


def time_batch(torch, lbm, lats, f0, steps, schedule):
    batch = lbm.DeviceBatch(lats, schedule=schedule)
    stream = torch.cuda.Stream()
    batch.set_stream(stream.cuda_stream)
    ns = [steps] * len(lats)
    best = float("inf")
    for rep in range(3):  # the first call captures the graph (graph path); the best of the rest counts
        for lat, f in zip(lats, f0):
            lat.upload(f)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        batch.step(ns)
        e1.record(stream)
        e1.synchronize()
        if rep:
            best = min(best, e0.elapsed_time(e1) / 1e3)
    batch.close()
    return best


def tune(members=8, steps=200, storages=STORAGES, quads=None, log=sys.stderr):
    import numpy as np
    import torch
    lbm = _package()
    lbm._native.lib()
    quads = quads or list(lbm.Quadratures)
    table = {"storages": {}, "measured_us_per_step": {}}
    for storage in storages:
        rows, meas = {}, {}
        for qn in quads:
            q = lbm.Quadratures[qn]
            per_q = {}
            best_rows = []
            for nx, ny in SHAPES:
                n = nx * ny
                lats = []
                for k in range(members):
                    lat = lbm.DeviceLattice(q, nx, ny, lbm.TRT.fields(0.8, 1.1), (), force=("constant", (1e-6, 0.0)),
                                            storage=storage)
                    lat.initialize_fields()
                    lats.append(lat)
                f0 = [lat.download() for lat in lats]
                res = {"graph": time_batch(torch, lbm, lats, f0, steps, None) / steps * 1e6}
                splits = SPLITS if storage in ("f64", "df64dev") and q.Q >= 9 else (1,)
                for per in PER_BLOCK:
                    if not resident_fits(q.Q, n, per, ELEM[storage]):
                        continue
                    for split in splits:
                        sched = {qn: {"resident_max_nodes": n, "nodes_per_block": per, "split": split}}
                        res[f"{per}x{split}"] = time_batch(torch, lbm, lats, f0, steps, sched) / steps * 1e6
                for lat in lats:
                    lat.close()
                per_q[str(n)] = {k: round(v, 3) for k, v in res.items()}
                best_rows.append((n, res))
                print(f"{storage} {qn} n={n}: " + ", ".join(f"{k} {v:.2f}" for k, v in res.items()) + " us/step",
                      file=log, flush=True)
            # the sizes up to the first one where no resident configuration beats the graph path
            wins = []
            for n, res in best_rows:
                if min((v for k, v in res.items() if k != "graph"), default=float("inf")) >= res["graph"]:
                    break
                wins.append((n, res))
            row = {"resident_max_nodes": 0, "nodes_per_block": 0, "split": 1}
            if wins:
                keys = [k for k in wins[-1][1] if k != "graph" and all(k in r for _, r in wins)]
                best = min(keys, key=lambda k: sum(r[k] / r["graph"] for _, r in wins))
                per, split = (int(v) for v in best.split("x"))
                row = {"resident_max_nodes": wins[-1][0], "nodes_per_block": per, "split": split}
            rows[qn] = row
            meas[qn] = per_q
        table["storages"][storage] = rows
        table["measured_us_per_step"][storage] = meas
    table["how"] = (f"tune_batch.py: {members} periodic TRT members per batch with a constant force, {steps} steps, "
                    "best of two timed calls after one untimed call, microseconds per global step; "
                    f"{torch.cuda.get_device_name(0)}, {time.strftime('%Y-%m-%d')}")
    return table


def main():
    table = tune()
    with open(os.path.join(HERE, "batch_schedule.json"), "w") as fh:
        json.dump(table, fh, indent=1, sort_keys=True)
    print(json.dumps(table["storages"], indent=1))


if __name__ == "__main__":
    main()
