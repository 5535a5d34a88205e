"""The simulate loop with the reference's processing methods, on the device, against the
oracle and against the reference's own printed results."""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
ROWS = json.load(open(os.path.join(HERE, "golden", "trt_magic_parameter_rows.json")))["rows"]


@pytest.mark.parametrize("row", ROWS[:4] + ROWS[-3:], ids=lambda r: f"{r['tau_s']}-{r['tau_a']}")
def test_reference_notebook_rows_on_gpu(lbm_gpu, row):
    """solve(problem, q, τ_s, τ_a) of examples/notebooks/trt_magic_parameter.ipynb through the
    GPU model: TRT with force, bounce-back walls, VelocityConvergence stop criterion."""
    lbm = lbm_gpu
    q = lbm.D2Q9()
    ts, ta = row["tau_s"], row["tau_a"]
    problem = lbm.PoiseuilleFlow((ts - 0.5) / q.speed_of_sound_squared, 1)
    n_steps = round(100.0 / problem.delta_t())
    pm = lbm.TrackHydrodynamicErrors(problem, False, n_steps, lbm.VelocityConvergenceStoppingCriteria(1e-7, problem))
    cm = lbm.TRT.fields(ts, ta, "problem")
    res = lbm.simulate(problem, q, t_end=100.0, should_process=False, collision_model=cm, process_method=pm,
                       initialization_strategy=lbm.ZeroVelocityInitialCondition())
    last = res.processing_method.df[-1]
    assert last.error_u == pytest.approx(row["error_u"], rel=6e-6)
    assert last.error_p == pytest.approx(row["error_p"], rel=6e-6)
    res.close()


def test_taylor_green_config_against_oracle(lbm_gpu, O):
    """D2Q9 SRT Taylor-Green vortex 64 x 64, τ = 0.8, equilibrium + off-equilibrium start,
    1000 steps, TrackHydrodynamicErrors at the last step: every field of the row."""
    lbm = lbm_gpu
    q = lbm.D2Q9()
    problem = lbm.TaylorGreenVortex(0.1, 1, 64, 64, static=False)
    pm = lbm.TrackHydrodynamicErrors(problem, False, 1000)
    m = lbm.LatticeBoltzmannModel(problem, q, collision_model=lbm.SRT,
                                  initialization_strategy=lbm.AnalyticalEquilibriumAndOffEquilibrium(),
                                  process_method=pm)
    lbm.simulate(m, time=range(0, 1000))
    row = pm.df[-1]
    op = O.taylor_green_vortex(0.1, 1, 64, 64, static=False)
    _, orows, _ = O.simulate("D2Q9", op, O.collision("SRT", [0.8]), [],
                             O.initialize(O.INIT_EQ_OFFEQ, "D2Q9", op), 0, 999, n_steps=1000)
    ref = orows[-1]
    assert row.timestep == ref["timestep"] == 1000
    # the error norms measure differences ~1e-4 of the fields: 1e-12 field parity gives ~1e-8 here
    for mine, key in [(row.error_ρ, "error_rho"), (row.error_u, "error_u"), (row.error_p, "error_p"),
                      (row.error_σ_xx, "error_sigma_xx"), (row.error_σ_xy, "error_sigma_xy")]:
        assert mine == pytest.approx(ref[key], rel=1e-7), key
    # mass and energy are O(1) sums; the total momentum is zero by symmetry up to rounding
    # noise (~1e-14 on 4096 nodes), compared on the scale of the mass
    assert row.mass == pytest.approx(ref["mass"], rel=1e-12)
    assert row.energy == pytest.approx(ref["energy"], rel=1e-9)
    assert abs(row.momentum - ref["momentum"]) <= 1e-12 * ref["mass"]
    m.close()


def test_compare_with_analytical_solution_and_mean_velocity_stop(lbm_gpu, O):
    """CompareWithAnalyticalSolution + MeanVelocityStoppingCriteria on a Couette flow
    (moving lid North, bounce-back South), every processed row against the oracle."""
    lbm = lbm_gpu
    q = lbm.D2Q9()
    problem = lbm.CouetteFlow(1.0 / 6.0, 2)
    pm = lbm.CompareWithAnalyticalSolution(problem, True, 400)
    m = lbm.LatticeBoltzmannModel(problem, q, collision_model=lbm.SRT, process_method=pm,
                                  initialization_strategy=lbm.ZeroVelocityInitialCondition())
    lbm.simulate(m, time=range(0, 400))
    op = O.couette(1.0 / 6.0, 2)
    obcs = [O.bc("bounce_back", "south", (1, 1), (1, op.ny)),
            O.bc("moving_wall", "north", (1, 1), (1, op.ny), u=(op.u_max, 0.0))]
    tau = 3.0 * (1.0 / 6.0) + 0.5
    _, orows, ostop = O.simulate("D2Q9", op, O.collision("SRT", [tau]), obcs,
                                 O.initialize(O.INIT_ZERO_VELOCITY, "D2Q9", op), 0, 399, pm_kind=O.PM_COMPARE,
                                 should_process=True, n_steps=400, stop_kind=O.STOP_MEAN_VELOCITY, stop_tol=1e-7)
    assert len(pm.df) == len(orows)
    for mine, ref in zip(pm.df, orows):
        for k in ["density", "momentum", "kinetic_energy", "internal_energy", "density_a", "momentum_a"]:
            assert getattr(mine, k) == pytest.approx(ref[k], rel=1e-10, abs=1e-15), k
    m.close()


def test_mei_iterative_initialisation_matches_oracle(lbm_gpu, O):
    """IterativeInitializationMeiEtAl on the device (DensityConvergence stop) against the oracle."""
    lbm = lbm_gpu
    q = lbm.D2Q9()
    problem = lbm.TaylorGreenVortex(0.1, 1, 16, 16, static=False)
    f = lbm.initialize(lbm.IterativeInitializationMeiEtAl(1.0, 1e-10), q, problem)
    op = O.taylor_green_vortex(0.1, 1, 16, 16, static=False)
    f0 = O.initialize(O.INIT_ZERO_VELOCITY, "D2Q9", op)
    fr, _, stopped = O.simulate("D2Q9", op, O.collision("ITER", [1.0]), [], f0, 1, 10000, pm_kind=O.PM_ITERATIVE,
                                stop_kind=O.STOP_DENSITY, stop_tol=1e-10, has_problem=False)
    assert stopped is not None
    np.testing.assert_allclose(f, fr, rtol=1e-12)


def test_snapshots(lbm_gpu, O):
    lbm = lbm_gpu
    q = lbm.D2Q9()
    problem = lbm.TaylorGreenVortex(0.1, 1, 16, 16, static=False)
    pm = lbm.TakeSnapshots(problem, [0, 5, 17])
    m = lbm.LatticeBoltzmannModel(problem, q, process_method=pm)
    f0 = m.f_stream
    lbm.simulate(m, time=range(0, 20))
    assert pm.timesteps == [5, 17]
    op = O.taylor_green_vortex(0.1, 1, 16, 16, static=False)
    dt = problem.delta_t()
    ref = O.run("D2Q9", op, O.collision("SRT", [0.8]), [], f0, 0, 16, dt=dt)
    np.testing.assert_allclose(pm.snapshots[1], ref, rtol=1e-12)
    m.close()
