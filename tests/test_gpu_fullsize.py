"""Full-size (4096 x 4096) D2Q9 TRT Poiseuille channel -- the benchmark workload -- checked
through size-independent properties: the flow is x-invariant, so every column equals the
oracle's run of a 3-column channel of the same height; all columns are bitwise equal; mass
is conserved by the periodic / bounce-back step."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NX = NY = 4096
STEPS = 60


def _channel(lbm, storage, tau_s=0.9):
    q = lbm.D2Q9()
    nu = (tau_s - 0.5) / q.speed_of_sound_squared
    u_max = 0.05
    problem = lbm.PoiseuilleFlow.fields(1.0, u_max, nu, NX, NY, 1.0, (1.0, 1.0), 1.0)
    # constant lattice force 1e-6 along x, as the benchmark configuration
    G = 1e-6 / (u_max * problem.delta_t() * problem.viscosity())
    problem.G = G
    cm = lbm.TRT.fields(tau_s, 0.5 + 0.25 / (tau_s - 0.5), "problem")
    m = lbm.LatticeBoltzmannModel(problem, q, collision_model=cm, storage=storage,
                                  initialization_strategy=lbm.ZeroVelocityInitialCondition())
    return problem, cm, m


@pytest.mark.parametrize("storage", ["f64", "df64dev"])
def test_fullsize_fp64_class_columns_match_oracle(lbm_gpu, O, storage):
    lbm = lbm_gpu
    problem, cm, m = _channel(lbm, storage)
    mass0 = m.lattice.conserved()[0]
    lbm.run_steps(m, 0, STEPS - 1)
    mass1 = m.lattice.conserved()[0]
    f = m.f_stream
    m.close()
    assert abs(mass1 - mass0) / mass0 < 1e-13
    for x in (1, 1000, NX - 1):
        assert np.array_equal(f[:, :, x], f[:, :, 0])
    p = O.poiseuille_struct(1.0, problem.u_max, problem.ν, 3, NY, 1.0, (1.0, 1.0), problem.G)
    ocm = O.collision("TRT", [cm.τ_symmetric, cm.τ_asymmetric], force=True)
    bcs = [O.bc("bounce_back", "north", (1, 3), (1, NY)), O.bc("bounce_back", "south", (1, 3), (1, NY))]
    ref = O.run("D2Q9", p, ocm, bcs, O.initialize(O.INIT_ZERO_VELOCITY, "D2Q9", p), 0, STEPS - 1,
                dt=problem.delta_t())
    err = np.max(np.abs(f[:, :, 0] - ref[:, :, 0]) / np.abs(ref[:, :, 0]))
    assert err <= 1e-12, err


def test_fullsize_f32dev_velocity_error(lbm_gpu):
    """FP32 deviation storage against FP64 on the forced channel.  Each step adds a near-constant
    force increment to values already on the FP32 grid, so round-to-nearest repeats the same
    rounding every step and the relative velocity error grows linearly in time (~1e-8 per step;
    3.6e-6 after 400 steps).  The float-float storage is the FP64-class path."""
    lbm = lbm_gpu
    res = {}
    for storage in ("f64", "f32dev"):
        _, _, m = _channel(lbm, storage)
        lbm.run_steps(m, 0, 399)
        rho, ux, uy = m.lattice.macroscopic()
        res[storage] = ux[:, 0].copy()
        m.close()
    rel = float(np.max(np.abs(res["f32dev"] - res["f64"])) / np.max(np.abs(res["f64"])))
    assert rel <= 1e-5, rel
