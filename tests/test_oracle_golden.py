"""The oracle against the reference's own printed outputs and against the oracle vectors
recorded when the oracle was validated (tests/golden/make_golden.py)."""
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROWS = json.load(open(os.path.join(HERE, "golden", "trt_magic_parameter_rows.json")))["rows"]
VECS = json.load(open(os.path.join(HERE, "golden", "oracle_vectors.json")))
TABLE = json.load(open(os.path.join(HERE, "golden", "trt_magic_parameter_table.json")))["rows"]


def _poiseuille_row(O, tau_s, tau_a):
    """solve(problem, q, τ_s, τ_a) of examples/notebooks/trt_magic_parameter.ipynb (cell 1)."""
    nu = (tau_s - 0.5) / 3.0
    p = O.poiseuille(nu, 1)
    dt = O.problem_scalars(p)["delta_t"]
    n_steps = round(100.0 / dt)
    cm = O.collision("TRT", [tau_s, tau_a], force=True)
    bcs = [O.bc("bounce_back", "north", (1, 3), (1, 5)), O.bc("bounce_back", "south", (1, 3), (1, 5))]
    f0 = O.initialize(O.INIT_ZERO_VELOCITY, "D2Q9", p)
    _, rows, _ = O.simulate("D2Q9", p, cm, bcs, f0, 0, n_steps, pm_kind=O.PM_TRACK, should_process=False,
                            n_steps=n_steps, stop_kind=O.STOP_VELOCITY, stop_tol=1e-7)
    return rows[-1]


@pytest.mark.parametrize("row", ROWS, ids=[f"{r['tau_s']}-{r['tau_a']}" for r in ROWS])
def test_oracle_reproduces_reference_notebook_rows(O, row):
    r = _poiseuille_row(O, row["tau_s"], row["tau_a"])
    # the notebook prints 6 significant digits
    assert r["error_u"] == pytest.approx(row["error_u"], rel=6e-6)
    assert r["error_p"] == pytest.approx(row["error_p"], rel=6e-6)


@pytest.mark.parametrize("row", TABLE, ids=[f"{r['tau_s']}-{r['tau_a']}" for r in TABLE])
def test_oracle_reproduces_reference_table_rows(O, row):
    """The notebook's 30-row HTML table, every printed column: error_u, error_p and error_σ_xy to
    the 6 printed digits, and error_σ_xx = Inf (the channel's analytic σ_xx is zero, and the
    reference divides by its norm, track_hydrodynamic_errors.jl:176-187)."""
    r = _poiseuille_row(O, float(row["tau_s"]), float(row["tau_a"]))
    assert row["quadrature"] == "D2Q9"
    assert r["error_u"] == pytest.approx(float(row["error_u"]), rel=6e-6)
    assert r["error_p"] == pytest.approx(float(row["error_p"]), rel=6e-6)
    assert r["error_sigma_xy"] == pytest.approx(float(row["error_sigma_xy"]), rel=6e-6)
    assert row["error_sigma_xx"] == "Inf" and r["error_sigma_xx"] == float("inf")


def test_oracle_vectors(O):
    p = O.poiseuille_struct(1.0, 0.1, 0.1, 3, 8, 1.0, (1.0, 1.0), 1.0)
    cm = O.collision("TRT", [0.8, 0.5 + 0.25 / 0.3], force=True)
    bcs = [O.bc("bounce_back", "north", (1, 3), (1, 8)), O.bc("bounce_back", "south", (1, 3), (1, 8))]
    f = O.run("D2Q9", p, cm, bcs, O.initialize(O.INIT_ZERO_VELOCITY, "D2Q9", p), 0, 49,
              dt=O.problem_scalars(p)["delta_t"])
    np.testing.assert_allclose(f[:, :, 1].ravel(), VECS["d2q9_trt_poiseuille_3x8_50"], rtol=1e-14)

    sw = O.shear_wave(6, 6, (0.6 - 0.5) / O.quadrature("D2Q37")["cs"])
    f = O.run("D2Q37", sw, O.collision("MRT", [0.6] * 4), [], O.initialize(O.INIT_EQUILIBRIUM, "D2Q37", sw), 0, 4)
    np.testing.assert_allclose(f[:, 2, 3], VECS["d2q37_mrt_shear_6x6_5"], rtol=1e-13)

    tg = O.taylor_green_vortex(0.1, 1, 16, 16, static=False)
    _, rows, _ = O.simulate("D2Q9", tg, O.collision("SRT", [0.8]), [], O.initialize(O.INIT_EQ_OFFEQ, "D2Q9", tg),
                            0, 40, n_steps=40)
    ref = VECS["d2q9_srt_tgv_16_40_row"]
    for k, v in rows[-1].items():
        assert v == pytest.approx(ref[k], rel=1e-11, abs=1e-300), k

    ld = O.lid_driven_cavity(1.0 / 6.0, 1, 7, 6)
    lbcs = [O.bc("bounce_back", "east", (1, 7), (1, 6)), O.bc("bounce_back", "south", (1, 7), (1, 6)),
            O.bc("bounce_back", "west", (1, 7), (1, 6)),
            O.bc("moving_wall", "north", (1, 7), (1, 6), u=(0.005, 0.0))]
    f = O.run("D2Q13", ld, O.collision("SRT", [1.0]), lbcs, O.initialize(O.INIT_EQUILIBRIUM, "D2Q13", ld), 0, 29)
    np.testing.assert_allclose(f[:, 5, 0], VECS["d2q13_srt_cavity_7x6_30"], rtol=1e-14)
