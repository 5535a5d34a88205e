"""Block-resident batched stepping (lbm_resident.cuh): members that the schedule makes resident
take all their steps of a call in one launch on a thread-block cluster, their populations in
shared memory and the pull crossing CTAs through distributed shared memory.  They must give
exactly what the graph path (one kernel per global step) gives: the same populations and the same
collision code, so bitwise for SRT / TRT and within rounding for MRT (both kernels collide an
array of populations with the same moment code; only the compiler's choice of fused multiply-adds
could differ between the two kernels).  Cluster sizes 1 to 8 are covered by the nodes-per-CTA
values, members smaller than their cluster (CTAs owning no node) included."""
import numpy as np
import pytest

from gpu_cases import rel_err, wave_field

pytestmark = pytest.mark.gpu

QUADS = ("D2Q4", "D2Q5", "D2Q9", "D2Q13", "D2Q17", "D2Q21", "D2Q37")

# (velocity set, nx, ny, steps per call, boundaries, force)
SPECS = [("D2Q9", 24, 3, 37, "walls", "constant"), ("D2Q37", 13, 9, 11, None, "field"),
         ("D2Q17", 5, 4, 23, "cavity", None), ("D2Q4", 1, 1, 5, None, None), ("D2Q21", 40, 24, 7, "walls", None),
         ("D2Q13", 7, 6, 0, None, None), ("D2Q5", 3, 2, 19, "walls", "constant"), ("D2Q9", 2, 3, 13, None, "field")]


def _bcs(lbm, kind, nx, ny):
    if kind == "walls":
        return [lbm.BounceBack(lbm.North(), (1, nx), (1, ny)), lbm.BounceBack(lbm.South(), (1, nx), (1, ny))]
    if kind == "cavity":
        return [lbm.BounceBack(lbm.East(), (1, nx), (1, ny)), lbm.BounceBack(lbm.South(), (1, nx), (1, ny)),
                lbm.BounceBack(lbm.West(), (1, nx), (1, ny)), lbm.MovingWall(lbm.North(), (1, nx), (1, ny), (0.01, 0.0))]
    return []


def _force(kind, nx, ny, seed):
    if kind == "constant":
        return ("constant", (1e-5, -2e-6))
    if kind == "field":
        rng = np.random.default_rng(seed)
        return ("field", 1e-5 * rng.normal(size=(2, ny, nx)))
    return None


def _models(lbm, storage, coll, specs=SPECS):
    out = []
    for k, (qn, nx, ny, _, bk, fk) in enumerate(specs):
        q = lbm.Quadratures[qn]
        cm = {"SRT": lbm.SRT(0.8), "TRT": lbm.TRT.fields(0.8, 1.15), "MRT": lbm.MRT(q, [0.8, 0.7, 1.1, 0.9])}[coll]
        out.append(lbm.LatticeBoltzmannModel.from_parts(q, wave_field(q, nx, ny, seed=500 + k, amp=0.01), cm,
                                                        _bcs(lbm, bk, nx, ny), force=_force(fk, nx, ny, k),
                                                        storage=storage))
    return out


def _resident(per, max_nodes=10 ** 9, split=1):
    return {q: {"resident_max_nodes": max_nodes, "nodes_per_block": per, "split": split} for q in QUADS}


def _run(lbm, storage, coll, schedule, specs=SPECS, calls=2):
    models = _models(lbm, storage, coll, specs)
    batch = lbm.DeviceBatch([m.lattice for m in models], schedule=schedule)
    steps = [s[3] for s in specs]
    for _ in range(calls):  # the first call starts from f_stream (collide-only first step), the next ones do not
        batch.step(steps)
    launches = batch.last_launch_count()
    batch.close()
    fs = [m.f_stream for m in models]
    for m in models:
        m.close()
    return fs, launches


def _same(fa, fb, coll, storage):
    for a, b, spec in zip(fa, fb, SPECS):
        if coll == "MRT":
            assert rel_err(a, b) <= (1e-6 if storage == "f32dev" else 1e-13), spec
        else:
            assert np.array_equal(a, b), spec


@pytest.mark.parametrize("storage", ["f64", "df64dev", "f32dev"])
@pytest.mark.parametrize("coll", ["SRT", "TRT", "MRT"])
@pytest.mark.parametrize("per", [8, 128])
@pytest.mark.parametrize("split", [1, 2, 4])
def test_resident_equals_graph_path(lbm_gpu, storage, coll, per, split):
    """split > 1 spreads each node's SRT / TRT collision over 2 or 4 warps where the library builds
    splits (FP64 and float-float from D2Q9 up); the other cases run unsplit."""
    lbm = lbm_gpu
    ref, graph_launches = _run(lbm, storage, coll, None)
    got, launches = _run(lbm, storage, coll, _resident(per, split=split))
    _same(got, ref, coll, storage)
    # graph: one kernel per global step of each velocity set's longest member; resident: one launch
    # per (velocity set, cluster size)
    assert graph_launches == 37 + 11 + 23 + 5 + 7 + 19
    assert launches <= len(QUADS) * 4


@pytest.mark.parametrize("storage", ["f64", "f32dev"])
def test_mixed_resident_and_graph_members(lbm_gpu, storage):
    """Members of at most 100 nodes resident, the others on the graph path, in one call."""
    lbm = lbm_gpu
    ref, _ = _run(lbm, storage, "TRT", None, calls=3)
    got, _ = _run(lbm, storage, "TRT", _resident(16, max_nodes=100), calls=3)
    _same(got, ref, "TRT", storage)


def test_resident_equals_solo_lattice(lbm_gpu):
    """A resident D2Q9 TRT channel with walls and a force, on a cluster of 4 CTAs, equals the
    lattice stepped alone through lbm_step (which the parity tests hold to the oracle)."""
    lbm = lbm_gpu
    spec = [("D2Q9", 24, 3, 37, "walls", "constant")]
    got, launches = _run(lbm, "f64", "TRT", _resident(18), specs=spec)
    assert launches == 1
    (m,) = _models(lbm, "f64", "TRT", spec)
    m.lattice.step(74, 0, 0.0)
    assert np.array_equal(got[0], m.f_stream)
    m.close()


SHEAR = [("D2Q9", 24, 3, 40, 5, 0.01), ("D2Q13", 17, 4, 25, 0, 0.02), ("D2Q9", 32, 5, 0, 3, 0.05),
         ("D2Q37", 16, 6, 31, 11, 0.003)]


def _shear_model(lbm, qname, nx, ny, storage, seed):
    q = lbm.Quadratures[qname]
    xr = (np.arange(nx) + 0.5) * 2 * np.pi / nx
    yr = (np.arange(ny) + 0.5) * 2 * np.pi / ny
    force = ("shear", [1e-4, 1.0, 0.3, 2e-4, 1.0, 0.7], xr, yr)
    return lbm.LatticeBoltzmannModel.from_parts(q, wave_field(q, nx, ny, seed=seed), lbm.SRT(0.8), force=force,
                                                storage=storage)


@pytest.mark.parametrize("storage", ["f64", "df64dev", "f32dev"])
@pytest.mark.parametrize("per,split", [(4, 1), (64, 1), (8, 4), (64, 2)])
def test_resident_time_dependent_force(lbm_gpu, storage, per, split):
    """Members with the time-dependent shear force, stepped with their own times: resident equals
    each lattice stepped alone through lbm_step (bitwise)."""
    lbm = lbm_gpu
    members = [_shear_model(lbm, q, nx, ny, storage, k) for k, (q, nx, ny, _, _, _) in enumerate(SHEAR)]
    solos = [_shear_model(lbm, q, nx, ny, storage, k) for k, (q, nx, ny, _, _, _) in enumerate(SHEAR)]
    steps = np.array([s[3] for s in SHEAR])
    t0 = np.array([s[4] for s in SHEAR])
    dt = np.array([s[5] for s in SHEAR])
    batch = lbm.DeviceBatch([m.lattice for m in members], schedule=_resident(per, split=split))
    batch.step(steps, t0, dt)
    batch.step(steps, t0 + steps, dt)
    batch.close()
    for (q, _, _, n, a, h), m, s in zip(SHEAR, members, solos):
        s.lattice.step(int(n), int(a), float(h))
        s.lattice.step(int(n), int(a + n), float(h))
        assert np.array_equal(m.f_stream, s.f_stream), (q, n)
        m.close()
        s.close()


def test_schedule_validation(lbm_gpu):
    lbm = lbm_gpu
    (m,) = _models(lbm, "f64", "SRT", [("D2Q9", 4, 4, 3, None, None)])
    batch = lbm.DeviceBatch([m.lattice])
    with pytest.raises(lbm._native.LbmError):
        batch.set_schedule({"D2Q9": {"resident_max_nodes": -1, "nodes_per_block": 8}})
    batch.set_schedule(None)
    batch.step([3])
    assert batch.last_launch_count() == 3  # graph path: one kernel per step
    batch.set_schedule(_resident(8))
    batch.step([3])
    assert batch.last_launch_count() == 1  # resident: one launch for all steps
    batch.close()
    m.close()
