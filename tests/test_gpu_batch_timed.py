"""Batches whose members carry a time-dependent force (LBM_FORCE_SHEAR, the static
DecayingShearFlow of decaying_shear_flow.jl:132-147): lbm_batch_step_timed steps member k at the
times (t0[k] + j) dt[k], exactly as lbm_step steps the lattice alone; the untimed call is refused.
And the reference's shear-wave convergence analysis (examples/notebooks/notebook_examples.jl:34-69)
run as one batch gives the rows of the sequential runs."""
import numpy as np
import pytest

from gpu_cases import wave_field

pytestmark = pytest.mark.gpu

SPECS = [("D2Q9", 24, 3, 40, 5, 0.01), ("D2Q13", 17, 4, 25, 0, 0.02), ("D2Q9", 32, 5, 0, 3, 0.05),
         ("D2Q17", 16, 6, 31, 11, 0.003)]


def _model(lbm, qname, nx, ny, storage, seed):
    q = lbm.Quadratures[qname]
    xr = (np.arange(nx) + 0.5) * 2 * np.pi / nx
    yr = (np.arange(ny) + 0.5) * 2 * np.pi / ny
    force = ("shear", [1e-4, 1.0, 0.3, 2e-4, 1.0, 0.7], xr, yr)
    return lbm.LatticeBoltzmannModel.from_parts(q, wave_field(q, nx, ny, seed=seed), lbm.SRT(0.8), force=force,
                                                storage=storage)


@pytest.mark.parametrize("storage", ["f64", "df64dev", "f32dev"])
def test_timed_batch_equals_individual_steps(lbm_gpu, storage):
    lbm = lbm_gpu
    N = lbm._native
    members = [_model(lbm, q, nx, ny, storage, k) for k, (q, nx, ny, _, _, _) in enumerate(SPECS)]
    solos = [_model(lbm, q, nx, ny, storage, k) for k, (q, nx, ny, _, _, _) in enumerate(SPECS)]
    steps = [s[3] for s in SPECS]
    t0 = np.array([s[4] for s in SPECS])
    dt = np.array([s[5] for s in SPECS])
    batch = lbm.DeviceBatch([m.lattice for m in members])
    with pytest.raises(N.LbmError):  # the members' times are required
        batch.step(steps)
    batch.step(steps, t0, dt)
    batch.step(steps, t0 + np.array(steps), dt)  # the cached graph again, from the advanced states
    batch.close()
    for (q, _, _, n, a, h), m, s in zip(SPECS, members, solos):
        s.lattice.step(n, a, h)
        s.lattice.step(n, a + n, h)
        assert np.array_equal(m.f_stream, s.f_stream), (q, n)
        m.close()
        s.close()


def test_shear_wave_study_batched_equals_sequential(lbm_gpu):
    import torch
    lbm = lbm_gpu
    res = lbm.run_shear_wave_study(("D2Q9", "D2Q17"), tau=0.8, scales=(1, 2, 4), torch=torch)
    assert res["max_rel_diff_batched_vs_sequential"] == 0.0
    assert 1.7 < res["orders"]["D2Q9"] < 2.5, res["orders"]


@pytest.mark.parametrize("storage", ["f64", "df64dev", "f32dev"])
@pytest.mark.parametrize("qname,nx", [("D2Q9", 24), ("D2Q17", 17)])
def test_time_dependent_force_in_graphs_equals_single_steps(lbm_gpu, storage, qname, nx):
    """lbm_step runs 64-step CUDA graphs also for a time-dependent force (each graph step reads
    its time from the device): 200 steps in one call, mostly graphs, equal 20 calls of 10
    steps, which never use a graph."""
    lbm = lbm_gpu
    a = _model(lbm, qname, nx, 6, storage, 1)
    b = _model(lbm, qname, nx, 6, storage, 1)
    t0, dt = 7, 0.013
    a.lattice.step(200, t0, dt)
    assert a.lattice.last_launch_count() == 200 + 3  # 3 graphs of 64 steps, each with its time advance
    for j in range(20):
        b.lattice.step(10, t0 + 10 * j, dt)
    assert np.array_equal(a.f_stream, b.f_stream)
    a.lattice.step(130, t0 + 200, dt)  # a second call: its graphs start from the new time
    for j in range(13):
        b.lattice.step(10, t0 + 200 + 10 * j, dt)
    assert np.array_equal(a.f_stream, b.f_stream)
    a.close()
    b.close()
