"""Batches of lattices (lbm_batch_*): one CUDA graph advancing lattices of different sizes,
velocity sets and step counts must give exactly what stepping each lattice alone gives, and
match the oracle."""
import numpy as np
import pytest

from gpu_cases import rel_err, wave_field

pytestmark = pytest.mark.gpu


def _members(lbm, storage):
    specs = [("D2Q9", 37, 21, "TRT", 25), ("D2Q17", 16, 16, "SRT", 9), ("D2Q9", 3, 5, "SRT", 40),
             ("D2Q13", 130, 3, "TRT", 1), ("D2Q9", 64, 48, "SRT", 0), ("D2Q17", 5, 4, "TRT", 17)]
    out = []
    for k, (qn, nx, ny, coll, steps) in enumerate(specs):
        q = lbm.Quadratures[qn]
        f0 = wave_field(q, nx, ny, seed=100 + k)
        cm = lbm.SRT(0.8) if coll == "SRT" else lbm.TRT.fields(0.8, 1.1)
        bcs = []
        force = None
        if k == 0:  # channel walls and a body force on one member
            bcs = [lbm.BounceBack(lbm.North(), (1, nx), (1, ny)), lbm.BounceBack(lbm.South(), (1, nx), (1, ny))]
            force = ("constant", (1e-5, 0.0))
        out.append((q, f0, cm, bcs, force, steps))
    return out


@pytest.mark.parametrize("storage", ["f64", "df64dev", "f32dev"])
def test_batch_equals_individual_steps(lbm_gpu, O, storage):
    lbm = lbm_gpu
    specs = _members(lbm, storage)
    # SRT and TRT cannot share one batch: group by collision kind
    for coll_kind in (lbm.SRT, lbm.TRT):
        group = [s for s in specs if isinstance(s[2], coll_kind)]
        batch_models = [lbm.LatticeBoltzmannModel.from_parts(q, f0, cm, bcs, force=force, storage=storage)
                        for q, f0, cm, bcs, force, _ in group]
        solo_models = [lbm.LatticeBoltzmannModel.from_parts(q, f0, cm, bcs, force=force, storage=storage)
                       for q, f0, cm, bcs, force, _ in group]
        steps = [s[5] for s in group]
        batch = lbm.DeviceBatch([m.lattice for m in batch_models])
        batch.step(steps)
        batch.step(steps)  # the second call replays the cached graph from the advanced states
        for m, n in zip(solo_models, steps):
            m.lattice.step(2 * n, 0, 0.0)
        for (q, f0, cm, bcs, force, n), mb, ms in zip(group, batch_models, solo_models):
            fb, fs = mb.f_stream, ms.f_stream
            assert np.array_equal(fb, fs), (q, n)
            if storage != "f32dev" and n > 0:
                p = O.lid_driven_cavity(1.0 / 6.0, 1, f0.shape[2], f0.shape[1])
                kind = "SRT" if isinstance(cm, lbm.SRT) else "TRT"
                taus = [cm.τ] if kind == "SRT" else [cm.τ_symmetric, cm.τ_asymmetric]
                obcs = [O.bc("bounce_back", b.direction.__class__.__name__.lower(), b.xs, b.ys) for b in bcs]
                if force is not None:
                    p = O.poiseuille_struct(1.0, 0.05, 0.1, f0.shape[2], f0.shape[1], 1.0, (1.0, 1.0), 1.0)
                    sc = O.problem_scalars(p)
                    p.G = force[1][0] / (p.u_max * sc["delta_t"] * sc["viscosity"])
                ref = O.run(q.name, p, O.collision(kind, taus, force=force is not None), obcs, f0, 0, 2 * n - 1,
                            dt=O.problem_scalars(p)["delta_t"] if force is not None else 0.0)
                assert rel_err(fb, ref) <= 1e-12, (q, n)
        batch.close()
        for m in batch_models + solo_models:
            m.close()


def test_small_tgv_convergence_study(lbm_gpu):
    """A reduced study (N = 16..128, D2Q9 and D2Q17): batched and sequential runs agree and
    the fitted velocity-error order is close to 2."""
    import torch
    lbm = lbm_gpu
    inst = lbm.tgv_instances(n_instances=16, sizes=(16, 32, 64, 128), tau_range=(0.8, 0.8),
                             steps_per_n2=1 / 64)
    res = lbm.run_tgv_study(inst, storage="df64dev", torch=torch)
    assert res["max_rel_diff_batched_vs_sequential"] == 0.0
    for q, order in res["orders"].items():
        assert 1.5 < order < 3.0, (q, order)


@pytest.mark.parametrize("storage", ["f64", "df64dev", "f32dev"])
@pytest.mark.parametrize("coll", ["SRT", "TRT", "MRT"])
def test_batch_every_velocity_set(lbm_gpu, storage, coll):
    """One batch of all seven velocity sets (MRT included), uneven sizes and step counts, equal
    to stepping each lattice alone: bitwise for SRT / TRT; for MRT to rounding, since the batched
    kernel collides an array of populations and the single-lattice kernel streams them through
    the same moment code, where the compiler may fuse multiply-adds differently."""
    lbm = lbm_gpu
    specs = [("D2Q4", 9, 7, 11), ("D2Q5", 12, 5, 3), ("D2Q9", 33, 20, 14), ("D2Q13", 17, 9, 0),
             ("D2Q17", 20, 11, 6), ("D2Q21", 7, 13, 9), ("D2Q37", 25, 18, 5)]
    models = {}
    for mode in ("batch", "solo"):
        ms = []
        for k, (qn, nx, ny, n) in enumerate(specs):
            q = lbm.Quadratures[qn]
            f0 = wave_field(q, nx, ny, seed=300 + k, amp=0.01)
            cm = {"SRT": lbm.SRT(0.75), "TRT": lbm.TRT.fields(0.75, 1.2), "MRT": lbm.MRT(q, 0.75)}[coll]
            ms.append(lbm.LatticeBoltzmannModel.from_parts(q, f0, cm, storage=storage))
        models[mode] = ms
    steps = np.array([s[3] for s in specs], dtype=np.int64)
    batch = lbm.DeviceBatch([m.lattice for m in models["batch"]])
    batch.step(steps)
    for m, n in zip(models["solo"], steps):
        m.lattice.step(int(n), 0, 0.0)
    for mb, ms, spec in zip(models["batch"], models["solo"], specs):
        if coll == "MRT":
            assert rel_err(mb.f_stream, ms.f_stream) <= (1e-7 if storage == "f32dev" else 1e-13), spec
        else:
            assert np.array_equal(mb.f_stream, ms.f_stream), spec
    batch.close()
    for m in models["batch"] + models["solo"]:
        m.close()
