"""Host-side logic of the studies and sweeps (no GPU): the points of the reference's TRT sweep,
the convergence-study instances, the order fit, and the shear-wave study's problem sizes and step
counts as notebook_examples.jl:34-69 defines them."""
import math

import numpy as np
import pytest


def test_julia_range_matches_the_notebook_grid(lbm):
    """range(0.51, stop = 10.0, step = 0.1) of trt_magic_parameter.ipynb: 95 decimal-exact points,
    each the double nearest 0.51 + 0.1 k (0.61, not 0.51 + 0.1 in binary)."""
    r = lbm.julia_range(0.51, 10.0, 0.1)
    assert len(r) == 95
    assert r[0] == 0.51 and r[1] == 0.61 and r[-1] == 9.91
    assert all(math.isclose(b - a, 0.1, rel_tol=1e-12) for a, b in zip(r, r[1:]))
    pts = lbm.trt_sweep_points(r)
    assert len(pts) == 95 * 95 and pts[0] == (0.51, 0.51) and pts[1] == (0.51, 0.61) and pts[95] == (0.61, 0.51)


def test_tgv_instances_are_seeded_round_robin(lbm):
    a = lbm.tgv_instances()
    b = lbm.tgv_instances()
    assert a == b and len(a) == 48
    pairs = [(n, q) for n in (16, 32, 64, 128, 256, 512, 1024) for q in ("D2Q9", "D2Q17")]
    for k, ins in enumerate(a):
        assert (ins["N"], ins["q"]) == pairs[k % len(pairs)]
        assert 0.51 <= ins["tau"] <= 2.0
        assert ins["steps"] == max(1, round(ins["N"] ** 2 / 256))
        assert ins["u0"] == pytest.approx(0.16 / ins["N"])


def test_convergence_order_of_exact_power_laws(lbm):
    inst = [{"N": n, "q": q} for q in ("D2Q9", "D2Q17") for n in (16, 32, 64, 128)]

    class Row:
        def __init__(self, e):
            self.error_u = e

    errors = [Row(3.0 * ins["N"] ** -2.0 if ins["q"] == "D2Q9" else 0.5 * ins["N"] ** -1.0) for ins in inst]
    orders = lbm.convergence_order(inst, errors)
    assert orders["D2Q9"] == pytest.approx(2.0, abs=1e-12)
    assert orders["D2Q17"] == pytest.approx(1.0, abs=1e-12)


@pytest.mark.parametrize("qname", ["D2Q9", "D2Q17", "D2Q37"])
def test_shear_wave_study_problems(lbm, qname):
    """DecayingShearFlow(ν, scale, static = true) with ν = τ / (2 speed_of_sound_squared): 8 scale x 3
    nodes (k_y = 0), n_steps = round(1 / Δt) growing like scale², and a force that depends on time."""
    q = lbm.Quadratures[qname]
    nu = 0.8 / (2.0 * q.speed_of_sound_squared)
    steps = []
    for scale in (1, 2, 4, 8):
        p = lbm.DecayingShearFlow(nu, scale, static=True)
        assert (p.NX, p.NY) == (8 * scale, 3)
        steps.append(int(round(1.0 / p.delta_t())))
        c = p.shear_force_params()
        assert c[5] != 0.0  # Fy = c3 cos(c4 x - c5 t): time enters the force
    ratios = np.array(steps[1:]) / np.array(steps[:-1])
    assert np.all(np.abs(ratios - 4.0) < 0.05), steps


def _track_row(lbm, e):
    vals = dict.fromkeys(lbm.processing_methods.TrackRow._fields, 0.0)
    vals.update(timestep=100, error_u=e, error_p=2 * e, error_σ_xx=3 * e, error_σ_xy=4 * e)
    return lbm.processing_methods.TrackRow(**vals)


def test_sweep_table_round_trip_and_grid(lbm, tmp_path):
    """The sweep's `results` table (trt_magic_parameter.ipynb cells 2-7): the seven columns in the
    loop's order, written and read back unchanged, and the τ_s x τ_a grid the contour plots."""
    taus = lbm.julia_range(0.51, 0.81, 0.1)
    pts = lbm.trt_sweep_points(taus)
    rows = {p: _track_row(lbm, p[0] * 10 + p[1]) for p in pts}
    table = lbm.trt_sweep_table(rows)
    assert tuple(table) == lbm.SWEEP_COLUMNS
    assert len(table["τ_s"]) == 16 and table["quadrature"][0] == "D2Q9"
    assert table["τ_s"][1] == 0.51 and table["τ_a"][1] == 0.61
    path = tmp_path / "trt_magic_parameter_001.npz"
    lbm.save_sweep_table(path, table)
    back = lbm.load_sweep_table(path)
    for c in lbm.SWEEP_COLUMNS:
        assert np.array_equal(back[c], table[c]), c
    ss, aa, grid = lbm.sweep_error_grid(back)
    assert list(ss) == taus and list(aa) == taus
    for ia, a in enumerate(aa):
        for js, s in enumerate(ss):
            assert grid[ia, js] == s * 10 + a
    _, _, gp = lbm.sweep_error_grid(back, "error_p")
    assert np.array_equal(gp, 2 * grid)


def test_sweep_table_gaps_and_errors(lbm, tmp_path):
    pts = [(0.6, 0.7), (0.8, 0.9)]
    table = lbm.trt_sweep_table({p: _track_row(lbm, 1.0) for p in pts}, quadrature="D2Q17")
    ss, aa, grid = lbm.sweep_error_grid(table)
    assert grid[0, 0] == 1.0 and grid[1, 1] == 1.0
    assert np.isnan(grid[0, 1]) and np.isnan(grid[1, 0])
    bad = dict(table)
    del bad["error_p"]
    with pytest.raises(ValueError):
        lbm.save_sweep_table(tmp_path / "x.npz", bad)
    bad = dict(table)
    bad["error_u"] = bad["error_u"][:1]
    with pytest.raises(ValueError):
        lbm.save_sweep_table(tmp_path / "y.npz", bad)
