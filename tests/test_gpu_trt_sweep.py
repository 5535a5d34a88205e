"""The TRT relaxation-time sweep of examples/notebooks/trt_magic_parameter.ipynb (cell 2: one
PoiseuilleFlow(ν, scale) run per (τ_s, τ_a), TRT with the lattice force, bounce-back walls,
velocity-convergence stop at 1e-7, t_end = 100) run as one device batch: every run's last
TrackHydrodynamicErrors row equals that of the same run simulated alone, and the results table
(cells 2-7) carries those rows."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("storage", ["f64", "df64dev"])
def test_batched_sweep_equals_sequential_runs(lbm_gpu, storage, tmp_path):
    import torch
    lbm = lbm_gpu
    taus = lbm.julia_range(0.51, 3.0, 0.5)
    pts = lbm.trt_sweep_points(taus)
    assert len(pts) == 25
    res = lbm.run_trt_sweep(pts, scale=1, storage=storage, sequential_points=pts, torch=torch)
    assert res["max_rel_diff_batched_vs_sequential"] == 0.0
    rows = res["rows"]
    assert list(rows) == pts
    for p, r in rows.items():
        assert r.timestep > 0 and math.isfinite(r.error_u), p
    table = lbm.trt_sweep_table(rows)
    path = tmp_path / "trt_sweep.npz"
    lbm.save_sweep_table(path, table)
    back = lbm.load_sweep_table(path)
    ss, aa, grid = lbm.sweep_error_grid(back)
    assert list(ss) == taus and list(aa) == taus
    for (ts, ta), r in rows.items():
        assert grid[taus.index(ta), taus.index(ts)] == r.error_u
    assert not np.isnan(grid).any()
