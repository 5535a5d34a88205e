"""The analytic Taylor-Green, Poiseuille and Couette solutions keep second-order convergence
through the GPU path (the reference's convergence studies: taylor_green_vortex.ipynb cell 3,
poiseuille.ipynb / trt_magic_parameter.ipynb `solve`, couette.ipynb), with every resolution of
a study run as one batch (simulate_batch)."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _order(ns, errs):
    return float(-np.polyfit(np.log(ns), np.log(errs), 1)[0])


@pytest.mark.parametrize("storage", ["f64", "df64dev"])
def test_taylor_green_second_order(lbm_gpu, storage):
    """TGV(q, τ, scale, 31 scale, 17 scale, u0 / scale) to its decay time, as the notebook."""
    lbm = lbm_gpu
    q = lbm.D2Q9()
    scales = [1, 2, 4]
    models, times = [], []
    for s in scales:
        problem = lbm.TGV(q, 0.8, s, 31 * s, 17 * s, math.sqrt(0.01) / s)
        t_end = round(lbm.decay_time(problem))
        pm = lbm.TrackHydrodynamicErrors(problem, False, t_end)
        models.append(lbm.LatticeBoltzmannModel(problem, q, process_method=pm, storage=storage,
                                                initialization_strategy=lbm.AnalyticalEquilibriumAndOffEquilibrium()))
        times.append(range(1, t_end + 1))
    lbm.simulate_batch(models, times)
    err = [m.processing_method.df[-1].error_u for m in models]
    for m in models:
        m.close()
    # the oracle gives 0.018840, 0.0043862, 0.0012954 (order 1.93)
    assert err == pytest.approx([0.018839581582715648, 0.004386156911387512, 0.0012953530075177527], rel=1e-9)
    assert 1.85 < _order(scales, err) < 2.1, err


def _channel_models(lbm, kind, scales, tau=0.8):
    q = lbm.D2Q9()
    nu = (tau - 0.5) / q.speed_of_sound_squared
    models, times = [], []
    for s in scales:
        problem = lbm.PoiseuilleFlow(nu, s) if kind == "poiseuille" else lbm.CouetteFlow(nu, s)
        n_steps = int(round(100.0 / problem.delta_t()))
        pm = lbm.TrackHydrodynamicErrors(problem, False, n_steps, lbm.VelocityConvergenceStoppingCriteria(1e-9, problem))
        cm = lbm.SRT(tau, "problem") if kind == "poiseuille" else lbm.SRT(tau)
        models.append(lbm.LatticeBoltzmannModel(problem, q, collision_model=cm, process_method=pm,
                                                initialization_strategy=lbm.ZeroVelocityInitialCondition()))
        times.append(range(0, n_steps + 1))
    return models, times


def test_poiseuille_second_order(lbm_gpu, O):
    """Steady Poiseuille flow (force, bounce-back walls), SRT τ = 0.8, run to the
    velocity-convergence stop as the notebooks' `solve` does: error_u falls by 4 per halving of
    Δx, and each row equals the oracle's."""
    lbm = lbm_gpu
    scales = [1, 2, 4, 8]
    models, times = _channel_models(lbm, "poiseuille", scales)
    lbm.simulate_batch(models, times)
    rows = [m.processing_method.df[-1] for m in models]
    for m in models:
        m.close()
    err = [r.error_u for r in rows]
    assert 1.9 < _order(scales, err) < 2.1, err
    nu = (0.8 - 0.5) / 3.0
    for s, r in zip(scales[:3], rows):
        p = O.poiseuille(nu, s)
        n_steps = int(round(100.0 / O.problem_scalars(p)["delta_t"]))
        bcs = [O.bc("bounce_back", "north", (1, p.nx), (1, p.ny)), O.bc("bounce_back", "south", (1, p.nx), (1, p.ny))]
        _, orows, stopped = O.simulate("D2Q9", p, O.collision("SRT", [0.8], force=True), bcs,
                                       O.initialize(0, "D2Q9", p), 0, n_steps, pm_kind=O.PM_TRACK, n_steps=n_steps,
                                       stop_kind=O.STOP_VELOCITY, stop_tol=1e-9)
        assert stopped == r.timestep
        assert r.error_u == pytest.approx(orows[-1]["error_u"], rel=1e-9)


def test_couette_is_exact(lbm_gpu):
    """Couette flow (moving lid, bounce-back floor) has a linear profile, which half-way
    bounce-back reproduces exactly: the error stays at the rounding level at every resolution."""
    lbm = lbm_gpu
    models, times = _channel_models(lbm, "couette", [1, 2, 4, 8])
    lbm.simulate_batch(models, times)
    err = [m.processing_method.df[-1].error_u for m in models]
    for m in models:
        m.close()
    assert all(e < 1e-9 for e in err), err


@pytest.mark.parametrize("storage", ["f64", "df64dev"])
@pytest.mark.parametrize("qname,coll,tau,expected", [
    ("D2Q9", "SRT", 0.8, [0.01025303463523784, 0.0025634013437757994, 0.0006408694124712757]),
    ("D2Q37", "MRT", 0.6, [0.031105040526872192, 0.007620077764117277, 0.0018956208479634419]),
])
def test_shear_wave_decay_second_order(lbm_gpu, storage, qname, coll, tau, expected):
    """Shear-wave decay u_x = u0 sin(2π y / N) exp(-ν k² t) (the D2Q37 regularised-MRT
    configuration's flow) over N = 16, 32, 64 with N²/16 steps, one batch: error_u equals the
    oracle's rows and falls with second order."""
    lbm = lbm_gpu
    q = lbm.Quadratures[qname]
    nu = (tau - 0.5) / q.speed_of_sound_squared
    sizes = [16, 32, 64]
    models, times = [], []
    for n in sizes:
        problem = lbm.ShearWave(n, n, nu, 0.01)
        steps = n * n // 16
        pm = lbm.TrackHydrodynamicErrors(problem, False, steps)
        cm = lbm.SRT(tau) if coll == "SRT" else lbm.MRT(q, tau)
        models.append(lbm.LatticeBoltzmannModel(problem, q, collision_model=cm, process_method=pm, storage=storage,
                                                initialization_strategy=lbm.AnalyticalEquilibrium()))
        times.append(range(0, steps))
    lbm.simulate_batch(models, times)
    err = [m.processing_method.df[-1].error_u for m in models]
    for m in models:
        m.close()
    assert err == pytest.approx(expected, rel=1e-9)
    assert 1.9 < _order(sizes, err) < 2.1
