"""CUDA path (liblbm_gb300 through its C ABI) against the CPU oracle, FP64-class storages.

The fused pull kernel is compared with the oracle's collide! -> stream! -> apply! loop on
the same inputs after N steps, for every velocity set, the SRT / TRT / regularised-MRT
collisions, periodic and bounce-back / moving-wall boundaries and every force kind.
Tolerance: max relative difference 1e-12 over all populations (the FP64 parity bound)."""
import numpy as np
import pytest

from gpu_cases import QUADS, rel_err, wave_field

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _run_pair(lbm, O, qname, nx, ny, coll, taus, steps, bcs_spec=(), force=None, f0=None, storage="f64"):
    q = lbm.Quadratures[qname]
    f0 = wave_field(q, nx, ny, seed=nx * 31 + ny) if f0 is None else f0
    if coll == "SRT":
        cm = lbm.SRT(taus[0])
    elif coll == "TRT":
        cm = lbm.TRT.fields(taus[0], taus[1])
    else:
        cm = lbm.MRT(q, list(taus))
    bcs, obcs = [], []
    for kind, d, xs, ys, u in bcs_spec:
        D = {"north": lbm.North(), "south": lbm.South(), "east": lbm.East(), "west": lbm.West()}[d]
        bcs.append(lbm.BounceBack(D, xs, ys) if kind == "bounce_back" else lbm.MovingWall(D, xs, ys, u))
        obcs.append(O.bc(kind, d, xs, ys, u=u))
    dev_force = None
    p = O.lid_driven_cavity(1.0 / 6.0, 1, nx, ny)
    ocm = O.collision(coll, taus, force=force is not None)
    if force == "constant":
        p = O.poiseuille_struct(1.0, 0.05, 0.1, nx, ny, 1.0, (1.0, 1.0), 1.0)
        F = O.force_field(p)
        dev_force = ("constant", (F[0, 0, 0], F[1, 0, 0]))
    elif force == "field":
        p = O.taylor_green_vortex(0.1, 1, nx, ny, static=True)
        dev_force = ("field", O.force_field(p))
    elif force == "shear":
        p = O.decaying_shear_flow(0.1, 1, nx, ny, static=True, k_y=1.0)
        sh = lbm.DecayingShearFlow(0.1, 1, nx, ny, static=True, k_y=1.0)
        xr, yr, _, _ = lbm.problem_range(sh)
        dev_force = ("shear", sh.shear_force_params(), xr, yr)
    dt = O.problem_scalars(p)["delta_t"] if force is not None else 0.0
    model = lbm.LatticeBoltzmannModel.from_parts(q, f0, cm, bcs, force=dev_force, storage=storage)
    model.lattice.step(steps, 0, dt)
    f_gpu = model.f_stream
    model.close()
    f_ref = O.run(qname, p, ocm, obcs, f0, 0, steps - 1, dt=dt)
    return f_gpu, f_ref


# the FP64-class storages, all held to the 1e-12 bound: FP64, the float-float deviation, and FP64
# storage with float-float arithmetic on the deviation
STORAGES = ["f64", "df64dev", "f64dd"]


@pytest.mark.parametrize("storage", STORAGES)
@pytest.mark.parametrize("qname", QUADS)
@pytest.mark.parametrize("coll,taus", [("SRT", [0.8]), ("TRT", [0.7, 1.1]), ("MRT", [0.9, 0.75, 1.2, 0.6])])
@pytest.mark.parametrize("nx", [37, 36])  # odd: one node per thread; even: the two-node packed kernel
def test_periodic(lbm_gpu, O, qname, coll, taus, storage, nx):
    f_gpu, f_ref = _run_pair(lbm_gpu, O, qname, nx, 21, coll, taus, 25, storage=storage)
    assert rel_err(f_gpu, f_ref) <= TOL


@pytest.mark.parametrize("storage", STORAGES)
@pytest.mark.parametrize("qname", QUADS)
@pytest.mark.parametrize("shape", [(1, 1), (2, 3), (5, 4), (130, 3)])
def test_small_and_ragged_lattices(lbm_gpu, O, qname, shape, storage):
    """Lattices smaller than the velocity set's reach (periodic wrap of |c| = 3 on a 1 x 1
    lattice, the reference's multispeed regression) and more than one x block."""
    f_gpu, f_ref = _run_pair(lbm_gpu, O, qname, shape[0], shape[1], "TRT", [0.8, 0.9], 7, storage=storage)
    assert rel_err(f_gpu, f_ref) <= TOL


def _walls(nx):
    return [("bounce_back", "north", (1, nx), (1, 16), (0.0, 0.0)),
            ("bounce_back", "south", (1, nx), (1, 16), (0.0, 0.0))]


def _cavity(nx):
    return [("bounce_back", "east", (1, nx), (1, 16), (0.0, 0.0)),
            ("bounce_back", "south", (1, nx), (1, 16), (0.0, 0.0)),
            ("bounce_back", "west", (1, nx), (1, 16), (0.0, 0.0)),
            ("moving_wall", "north", (1, nx), (1, 16), (0.004, 0.0))]


def _partial(nx):
    return [("bounce_back", "north", (3, 11), (14, 16), (0.0, 0.0)),
            ("bounce_back", "west", (1, 2), (5, 9), (0.0, 0.0)),
            ("bounce_back", "south", (1, nx), (1, 1), (0.0, 0.0))]


WALLS = _walls(19)


@pytest.mark.parametrize("storage", STORAGES)
@pytest.mark.parametrize("qname", QUADS)
@pytest.mark.parametrize("bcs", [_walls, _cavity, _partial], ids=["walls", "cavity", "partial"])
@pytest.mark.parametrize("coll,taus", [("SRT", [0.9]), ("TRT", [0.8, 1.05]), ("MRT", [0.8, 0.8, 0.8, 0.8])])
@pytest.mark.parametrize("nx", [19, 20])  # odd: one node per thread; even: the two-node packed kernel
def test_boundaries(lbm_gpu, O, qname, bcs, coll, taus, storage, nx):
    f_gpu, f_ref = _run_pair(lbm_gpu, O, qname, nx, 16, coll, taus, 20, bcs_spec=bcs(nx), storage=storage)
    assert rel_err(f_gpu, f_ref) <= TOL


@pytest.mark.parametrize("storage", STORAGES)
@pytest.mark.parametrize("qname", ["D2Q9", "D2Q17", "D2Q37"])
@pytest.mark.parametrize("force", ["constant", "field", "shear"])
@pytest.mark.parametrize("coll,taus", [("SRT", [0.8]), ("TRT", [0.8, 0.95]), ("MRT", [0.7, 0.9, 0.7, 0.7])])
def test_forces(lbm_gpu, O, qname, force, coll, taus, storage):
    bcs = WALLS if force == "constant" else ()
    nx, ny = (19, 16) if force == "constant" else (16, 16)
    f_gpu, f_ref = _run_pair(lbm_gpu, O, qname, nx, ny, coll, taus, 20, bcs_spec=bcs, force=force,
                             storage=storage)
    assert rel_err(f_gpu, f_ref) <= TOL


def test_determinism(lbm_gpu):
    """Two identical runs give bitwise identical populations."""
    lbm = lbm_gpu
    q = lbm.D2Q9()
    f0 = wave_field(q, 64, 48, seed=3)
    outs = []
    for _ in range(2):
        m = lbm.LatticeBoltzmannModel.from_parts(q, f0, lbm.TRT.fields(0.8, 1.0))
        m.lattice.step(100, 0, 0.0)
        outs.append(m.f_stream)
        m.close()
    assert np.array_equal(outs[0], outs[1])
