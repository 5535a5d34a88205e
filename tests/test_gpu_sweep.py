"""Batched time loops (simulate_batch over a DeviceBatch with batched stop-criterion
reductions): the TRT relaxation-time sweep of examples/notebooks/trt_magic_parameter.ipynb."""
import json
import os

import numpy as np
import pytest

from gpu_cases import wave_field

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROWS = json.load(open(os.path.join(HERE, "golden", "trt_magic_parameter_rows.json")))["rows"]
TABLE = json.load(open(os.path.join(HERE, "golden", "trt_magic_parameter_table.json")))["rows"]


def test_batched_sweep_reproduces_the_notebook_rows(lbm_gpu):
    """All 21 printed rows of the notebook, as ONE batch: error_u and error_p to the printed digits."""
    lbm = lbm_gpu
    points = [(r["tau_s"], r["tau_a"]) for r in ROWS]
    models, times = lbm.build_trt_sweep_models(points, scale=1)
    lbm.simulate_batch(models, times)
    for r, m in zip(ROWS, models):
        last = m.processing_method.df[-1]
        assert last.error_u == pytest.approx(r["error_u"], rel=6e-6), r
        assert last.error_p == pytest.approx(r["error_p"], rel=6e-6), r
        m.close()


def test_batched_sweep_reproduces_the_notebook_table(lbm_gpu):
    """The notebook's 30-row HTML table as ONE batch, every printed column: error_u, error_p and
    error_σ_xy to the printed digits, error_σ_xx = Inf (zero analytic σ_xx)."""
    lbm = lbm_gpu
    points = [(float(r["tau_s"]), float(r["tau_a"])) for r in TABLE]
    models, times = lbm.build_trt_sweep_models(points, scale=1)
    lbm.simulate_batch(models, times)
    for r, m in zip(TABLE, models):
        last = m.processing_method.df[-1]
        assert last.error_u == pytest.approx(float(r["error_u"]), rel=6e-6), r
        assert last.error_p == pytest.approx(float(r["error_p"]), rel=6e-6), r
        assert last.error_σ_xy == pytest.approx(float(r["error_sigma_xy"]), rel=6e-6), r
        assert r["error_sigma_xx"] == "Inf" and last.error_σ_xx == float("inf"), r
        m.close()


def test_batched_sweep_equals_sequential(lbm_gpu):
    """Runs that stop early, run to n_steps or blow up: every row field of every run is the same
    batched and one after another (same kernels, same reduction order)."""
    lbm = lbm_gpu
    points = lbm.trt_sweep_points([0.51, 0.8, 1.7, 6.0], [0.51, 0.6, 1.3, 9.0])
    res = {}
    for mode in ("batched", "sequential"):
        models, times = lbm.build_trt_sweep_models(points, scale=2)
        if mode == "batched":
            lbm.simulate_batch(models, times)
        else:
            for m, tm in zip(models, times):
                lbm.simulate_model(m, tm)
        res[mode] = [list(m.processing_method.df) for m in models]
        for m in models:
            m.close()
    for a, b in zip(res["batched"], res["sequential"]):
        assert len(a) == len(b)
        for ra, rb in zip(a, b):
            np.testing.assert_array_equal(np.array(ra, dtype=float), np.array(rb, dtype=float))


def _lattices(lbm, storage):
    out = []
    for qname, nx, ny, seed in (("D2Q9", 40, 24, 1), ("D2Q13", 33, 17, 2), ("D2Q9", 5, 3, 3)):
        q = lbm.Quadratures[qname]
        f0 = wave_field(q, nx, ny, seed=seed, amp=0.01)
        cm = lbm.TRT.fields(0.8, 1.1)
        m = lbm.LatticeBoltzmannModel.from_parts(q, f0, cm, storage=storage)
        out.append(m)
    return out


@pytest.mark.parametrize("storage", ["f64", "df64dev", "f32dev"])
def test_batch_reduce_matches_single_lattice_reduce(lbm_gpu, storage):
    lbm = lbm_gpu
    N = lbm._native
    A, B = _lattices(lbm, storage), _lattices(lbm, storage)
    batch = lbm.DeviceBatch([m.lattice for m in A])
    batch.step(np.array([7, 3, 0], dtype=np.int64))
    for m, k in zip(B, (7, 3, 0)):
        m.lattice.step(k, 0, 0.0)
    for kind in (N.REDUCE_MEAN_VELOCITY, N.REDUCE_CONSERVED):
        rows = batch.reduce(kind)
        for k, m in enumerate(B):
            np.testing.assert_array_equal(rows[k], m.lattice.reduce(kind)[: rows.shape[1]])
    # velocity convergence updates the previous-velocity planes of the selected members only
    sel = np.array([1, 0, 1], dtype=np.uint8)
    for _ in range(2):
        rows = batch.reduce(N.REDUCE_VELOCITY_CONVERGENCE, sel)
        for k, m in enumerate(B):
            if sel[k]:
                np.testing.assert_array_equal(rows[k], m.lattice.reduce(N.REDUCE_VELOCITY_CONVERGENCE))
            else:
                assert not rows[k].any()
    np.testing.assert_array_equal(batch.reduce(N.REDUCE_VELOCITY_CONVERGENCE)[1],
                                  B[1].lattice.reduce(N.REDUCE_VELOCITY_CONVERGENCE))
    batch.close()
    for m in A + B:
        m.close()


def _mixed_models(lbm):
    """Runs with MeanVelocity stop criteria (the reference's defaults for Poiseuille and Couette),
    TrackHydrodynamicErrors and CompareWithAnalyticalSolution, uneven sizes and run lengths."""
    q = lbm.D2Q9()
    models, times = [], []
    for k, (nu, scale) in enumerate([(0.05, 1), (0.1, 2), (0.3, 1), (0.8, 2), (0.02, 1)]):
        for kind in ("poiseuille", "couette"):
            problem = (lbm.PoiseuilleFlow(nu, scale) if kind == "poiseuille" else lbm.CouetteFlow(nu, scale))
            n_steps = int(round(5.0 / problem.delta_t()))
            pm = (lbm.TrackHydrodynamicErrors(problem, False, n_steps) if k % 2 == 0
                  else lbm.CompareWithAnalyticalSolution(problem, False, n_steps))
            models.append(lbm.LatticeBoltzmannModel(problem, q, collision_model=lbm.TRT, process_method=pm,
                                                    initialization_strategy=lbm.ZeroVelocityInitialCondition()))
            times.append(range(0, n_steps + 1))
    return models, times


def test_batched_mean_velocity_and_compare_equal_sequential(lbm_gpu):
    lbm = lbm_gpu
    res = {}
    for mode in ("batched", "sequential"):
        models, times = _mixed_models(lbm)
        if mode == "batched":
            lbm.simulate_batch(models, times)
        else:
            for m, tm in zip(models, times):
                lbm.simulate_model(m, tm)
        res[mode] = [(list(m.processing_method.df), m.processing_method.stop_criteria.old_mean_velocity)
                     for m in models]
        for m in models:
            m.close()
    for (ra, oa), (rb, ob) in zip(res["batched"], res["sequential"]):
        assert oa == ob
        assert len(ra) == len(rb) and len(ra) >= 1
        for a, b in zip(ra, rb):
            np.testing.assert_array_equal(np.array(a, dtype=float), np.array(b, dtype=float))


def test_batched_generic_path_every_step_processing(lbm_gpu):
    """should_process = true (a row every step) takes the per-member path of simulate_batch."""
    lbm = lbm_gpu
    res = {}
    for mode in ("batched", "sequential"):
        q = lbm.D2Q9()
        models = []
        for nx in (16, 24, 8):
            problem = lbm.TaylorGreenVortex(0.1, 1, nx, nx, static=False)
            pm = lbm.TrackHydrodynamicErrors(problem, True, 60)
            models.append(lbm.LatticeBoltzmannModel(problem, q, collision_model=lbm.SRT, process_method=pm))
        times = [range(0, 40), range(0, 60), range(0, 25)]
        if mode == "batched":
            lbm.simulate_batch(models, times)
        else:
            for m, tm in zip(models, times):
                lbm.simulate_model(m, tm)
        res[mode] = [list(m.processing_method.df) for m in models]
        for m in models:
            m.close()
    for a, b in zip(res["batched"], res["sequential"]):
        assert len(a) == len(b)
        for ra, rb in zip(a, b):
            np.testing.assert_array_equal(np.array(ra, dtype=float), np.array(rb, dtype=float))


@pytest.mark.parametrize("storage", ["f64", "df64dev", "f32dev"])
def test_batch_field_reductions_match_single_lattice(lbm_gpu, storage):
    """lbm_batch_reduce_fields (TRACK_ERRORS, COMPARE with per-member analytic planes) gives
    bitwise the sums lbm_reduce gives for each member."""
    lbm = lbm_gpu
    N = lbm._native
    A = _lattices(lbm, storage)
    batch = lbm.DeviceBatch([m.lattice for m in A])
    batch.step(np.array([5, 2, 0], dtype=np.int64))
    rng = np.random.default_rng(5)
    inputs = []
    for k, m in enumerate(A):
        lat = m.lattice
        fields = {name: rng.normal(size=(lat.ny, lat.nx)) * 1e-2 + (1.0 if name == "rho" else 0.0)
                  for name in ("rho", "ux", "uy", "p", "sxx", "syx", "sxy", "syy")}
        inputs.append(None if k == 1 else (fields, 0.3 + 0.1 * k, 0.05, 0.25))
    for kind in (N.REDUCE_TRACK_ERRORS, N.REDUCE_COMPARE):
        rows = batch.reduce_fields(kind, inputs)
        for k, m in enumerate(A):
            if inputs[k] is None:
                assert not rows[k].any()
                continue
            fields, tau, u_max, area = inputs[k]
            single = m.lattice.reduce(kind, fields, tau=tau, u_max=u_max, area=area)
            np.testing.assert_array_equal(rows[k], single)
    batch.close()
    for m in A:
        m.close()
