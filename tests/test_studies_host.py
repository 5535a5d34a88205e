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
