"""The two-node packed step (deviation storages, SRT and TRT, even nx) against the one-node
collision.  A batch runs the one-node collision on every member, so a lattice stepped alone (the
packed kernel, for even nx) must equal the same lattice stepped in a batch bitwise — with
bounce-back walls on every side and a moving wall (whose rows and columns take the kernel's general
pull), with a constant, a per-node and a time-dependent force; the last is also checked against
the FP64 run."""
import numpy as np
import pytest

from gpu_cases import wave_field

pytestmark = pytest.mark.gpu

SETS = ["D2Q4", "D2Q5", "D2Q9", "D2Q13", "D2Q17", "D2Q21"]
CASES = ["walls_constant", "moving_wall_field", "side_walls", "walls_shear"]


def _case(lbm, case, nx, ny, rng):
    N, S, E, W = lbm.North(), lbm.South(), lbm.East(), lbm.West()
    if case == "walls_constant":
        return [lbm.BounceBack(N, (1, nx), (1, ny)), lbm.BounceBack(S, (1, nx), (1, ny))], \
            ("constant", (2e-5, -1e-5))
    if case == "moving_wall_field":
        ff = 1e-5 * rng.normal(size=(2, ny, nx))
        return [lbm.BounceBack(S, (1, nx), (1, ny)), lbm.MovingWall(N, (1, nx), (1, ny), (0.02, 0.0))], \
            ("field", ff)
    if case == "walls_shear":
        xr = (np.arange(nx) + 0.5) / nx
        yr = (np.arange(ny) + 0.5) / ny
        return [lbm.BounceBack(N, (1, nx), (1, ny)), lbm.BounceBack(S, (1, nx), (1, ny))], \
            ("shear", [1e-5, 2 * np.pi, 0.01, 2e-5, 2 * np.pi, 0.02], xr, yr)
    return [lbm.BounceBack(W, (1, nx), (1, ny)), lbm.BounceBack(E, (1, nx), (1, ny))], None


@pytest.mark.parametrize("storage", ["f32dev", "df64dev"])
@pytest.mark.parametrize("qname", SETS)
@pytest.mark.parametrize("case", CASES)
def test_packed_step_equals_one_node_collision(lbm_gpu, storage, qname, case):
    lbm = lbm_gpu
    q = lbm.Quadratures[qname]
    nx, ny, steps = 24, 14, 23
    rng = np.random.default_rng(SETS.index(qname) * 10 + CASES.index(case))
    f0 = wave_field(q, nx, ny, seed=7)
    bcs, force = _case(lbm, case, nx, ny, rng)
    for cm in (lbm.SRT(0.8), lbm.TRT.fields(0.8, 1.1)):
        solo = lbm.LatticeBoltzmannModel.from_parts(q, f0, cm, bcs, force=force, storage=storage)
        member = lbm.LatticeBoltzmannModel.from_parts(q, f0, cm, bcs, force=force, storage=storage)
        batch = lbm.DeviceBatch([member.lattice])
        solo.lattice.step(steps, 3, 0.5)
        batch.step([steps], [3], [0.5])
        fs, fb = solo.f_stream, member.f_stream
        batch.close()
        solo.close()
        member.close()
        assert np.all(np.isfinite(fs))
        assert np.array_equal(fs, fb), (qname, case, type(cm).__name__, float(np.max(np.abs(fs - fb))))


@pytest.mark.parametrize("storage,tol", [("f32dev", 1e-5), ("df64dev", 1e-9), ("f16dev", 5e-2)])
@pytest.mark.parametrize("qname", ["D2Q9", "D2Q17"])
def test_packed_step_with_shear_force(lbm_gpu, storage, tol, qname):
    lbm = lbm_gpu
    q = lbm.Quadratures[qname]
    nx, ny = 32, 20
    f0 = wave_field(q, nx, ny, seed=5, amp=0.01)
    xr = (np.arange(nx) + 0.5) / nx
    yr = (np.arange(ny) + 0.5) / ny
    force = ("shear", [1e-5, 2 * np.pi, 0.01, 2e-5, 2 * np.pi, 0.02], xr, yr)
    out = {}
    for st in ("f64", storage):
        m = lbm.LatticeBoltzmannModel.from_parts(q, f0, lbm.TRT.fields(0.8, 1.0), force=force, storage=st)
        m.lattice.step(60, 0, 0.5)
        out[st] = m.lattice.macroscopic()
        m.close()
    u64 = np.hypot(out["f64"][1], out["f64"][2])
    du = np.hypot(out[storage][1] - out["f64"][1], out[storage][2] - out["f64"][2])
    assert float(du.max() / u64.max()) < tol
