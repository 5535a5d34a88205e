"""Initial conditions built on the device from macroscopic planes (lbm_initialize_fields)
against the host construction `initialize(strategy, q, problem)` (initial_conditions.jl and
initial_conditions/*.jl restated in numpy)."""
import numpy as np
import pytest

from gpu_cases import QUADS

pytestmark = pytest.mark.gpu

STRATEGIES = ["ZeroVelocityInitialCondition", "AnalyticalEquilibrium", "AnalyticalEquilibriumAndOffEquilibrium",
              "ConstantDensity", "AnalyticalVelocityAndStress"]


def _problems(lbm, q):
    yield "TaylorGreenVortex", lbm.TaylorGreenVortex(0.1, 1, 24, 20, static=False)
    yield "TGV", lbm.TGV(q, 0.9, 1, 16, 12, 0.02)
    yield "DecayingShearFlow", lbm.DecayingShearFlow(0.1, 1, 12, 16, static=False)
    yield "LinearizedThermalDiffusion", lbm.LinearizedThermalDiffusion(0.1, 0.1, 1, 16)
    yield "PoiseuilleFlow", lbm.PoiseuilleFlow(0.1, 2)


@pytest.mark.parametrize("qname", QUADS)
@pytest.mark.parametrize("strategy", STRATEGIES)
@pytest.mark.parametrize("storage", ["f64", "df64dev", "f32dev"])
def test_device_initialisation_matches_host(lbm_gpu, qname, strategy, storage):
    lbm = lbm_gpu
    q = lbm.Quadratures[qname]
    st = getattr(lbm, strategy)()
    for name, problem in _problems(lbm, q):
        try:
            host = lbm.initialize(st, q, problem)
        except (NotImplementedError, AttributeError, TypeError):
            continue  # the combination has no initial condition in the reference either
        m = lbm.LatticeBoltzmannModel(problem, q, collision_model=lbm.SRT(0.8), initialization_strategy=st,
                                      storage=storage, device_init=True)
        dev = m.f_stream
        m.close()
        scale = float(np.max(np.abs(host)))
        err = float(np.max(np.abs(dev - host))) / scale
        tol = {"f64": 1e-13, "df64dev": 1e-13, "f32dev": 1e-7}[storage]
        assert err <= tol, (name, err)


def test_device_initialisation_default_path(lbm_gpu):
    """The model builds closed-form initial conditions on the device by default and uploads the
    host array only for explicit f0 or device_init=False."""
    lbm = lbm_gpu
    q = lbm.D2Q9()
    problem = lbm.TaylorGreenVortex(0.1, 1, 32, 32, static=False)
    st = lbm.AnalyticalEquilibriumAndOffEquilibrium()
    a = lbm.LatticeBoltzmannModel(problem, q, initialization_strategy=st)
    b = lbm.LatticeBoltzmannModel(problem, q, initialization_strategy=st, device_init=False)
    fa, fb = a.f_stream, b.f_stream
    assert np.max(np.abs(fa - fb)) <= 1e-15
    lbm.simulate(a, time=range(0, 50))
    lbm.simulate(b, time=range(0, 50))
    assert np.max(np.abs(a.f_stream - b.f_stream)) <= 1e-14
    a.close()
    b.close()
