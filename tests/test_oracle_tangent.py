"""The oracle's forward-mode derivative (dual numbers through the same collide / stream
templates as its double loop; the stand-in for ForwardDiff through the reference, which types
τ as Float64 in srt.jl:2): its value part is the double loop, its derivative part agrees with
central differences of that loop.  CPU only."""
import numpy as np
import pytest

NX, NY, STEPS = 12, 10, 30


def _fields(lbm, nx=NX, ny=NY):
    u0 = lbm.divergence_free_field(nx, ny, kmax=3, amplitude=0.01, seed=11)
    ut = lbm.divergence_free_field(nx, ny, kmax=3, amplitude=0.01, seed=12)
    return u0, ut


def _double_loop_loss(O, q, kind, taus, u0, ut, steps):
    """The loss from the oracle's own double loop (orc_run: collide -> stream, no force)."""
    Q = O.quadrature(q)
    _, ny, nx = u0.shape
    f0 = np.empty((Q["Q"], ny, nx))
    for y in range(ny):
        for x in range(nx):
            f0[:, y, x] = O.equilibrium(q, 1.0, (u0[0, y, x], u0[1, y, x]))
    p = O.poiseuille_struct(1.0, 0.05, 0.1, nx, ny, 1.0, (1.0, 1.0), 0.0)
    f = O.run(q, p, O.collision(kind, list(taus), force=False), [], f0, 0, steps - 1)
    cx, cy = np.array(Q["cx"], dtype=float), np.array(Q["cy"], dtype=float)
    rho = f.sum(axis=0)
    ux = np.tensordot(cx, f, 1) / rho
    uy = np.tensordot(cy, f, 1) / rho
    return float(np.sum((ux - ut[0]) ** 2 + (uy - ut[1]) ** 2))


@pytest.mark.parametrize("q,kind", [("D2Q9", "TRT"), ("D2Q9", "SRT"), ("D2Q13", "TRT"), ("D2Q9", "MRT"),
                                    ("D2Q13", "MRT")])
def test_value_part_is_the_double_loop(lbm, O, q, kind):
    u0, ut = _fields(lbm)
    taus = (0.8, 1.1)
    L, _ = O.tangent_loss(q, kind, taus, (0.0, 0.0), u0, ut, STEPS, seed=(1.0, 0.0, 0.0, 0.0))
    assert L == pytest.approx(_double_loop_loss(O, q, kind, taus, u0, ut, STEPS), rel=1e-13)


@pytest.mark.parametrize("q,kind", [("D2Q9", "TRT"), ("D2Q9", "SRT"), ("D2Q13", "TRT"), ("D2Q9", "MRT"),
                                    ("D2Q13", "MRT")])
def test_tangents_match_central_differences(lbm, O, q, kind):
    u0, ut = _fields(lbm)
    taus, F = [0.8, 1.1], [2e-6, -1e-6]
    v = np.random.default_rng(5).normal(size=u0.shape)

    def value(dt0=0.0, dt1=0.0, dfx=0.0, dfy=0.0, du=0.0):
        return O.tangent_loss(q, kind, (taus[0] + dt0, taus[1] + dt1), (F[0] + dfx, F[1] + dfy), u0 + du * v, ut,
                              STEPS)[0]

    def fd(fun, h):
        return (fun(-2 * h) - 8 * fun(-h) + 8 * fun(h) - fun(2 * h)) / (12 * h)

    checks = [((1, 0, 0, 0), None, fd(lambda e: value(dt0=e), 1e-4)),
              ((0, 0, 1, 0), None, fd(lambda e: value(dfx=e), 1e-7)),
              ((0, 0, 0, 1), None, fd(lambda e: value(dfy=e), 1e-7)),
              ((0, 0, 0, 0), v, fd(lambda e: value(du=e), 1e-5))]
    if kind in ("TRT", "MRT"):  # MRT of a second-order set: the outputs depend on τs[2] only
        checks.append(((0, 1, 0, 0), None, fd(lambda e: value(dt1=e), 1e-4)))
    for seed, du0, ref in checks:
        _, d = O.tangent_loss(q, kind, taus, F, u0, ut, STEPS, seed=seed, du0=du0)
        assert d == pytest.approx(ref, rel=1e-6, abs=1e-13), (seed, d, ref)


def _walls(O, nx=NX, ny=NY, lid=False):
    out = [O.bc("bounce_back", "north", (1, nx), (1, ny)), O.bc("bounce_back", "south", (1, nx), (1, ny))]
    if lid:
        out = [O.bc("bounce_back", "east", (1, nx), (1, ny)), O.bc("bounce_back", "south", (1, nx), (1, ny)),
               O.bc("bounce_back", "west", (1, nx), (1, ny)),
               O.bc("moving_wall", "north", (1, nx), (1, ny), u=(0.01, 0.0))]
    return out


@pytest.mark.parametrize("lid", [False, True])
def test_walled_value_part_is_the_double_loop(lbm, O, lid):
    """With bounce-back walls (and a moving lid) after the periodic stream, the dual loop's value
    part is the oracle's double loop with the same boundary list (bounce_back.jl:8-72)."""
    u0, ut = _fields(lbm)
    q, taus = "D2Q9", (0.8, 1.1)
    bcs = _walls(O, lid=lid)
    L, _ = O.tangent_loss(q, "TRT", taus, (0.0, 0.0), u0, ut, STEPS, seed=(1.0, 0.0, 0.0, 0.0), bcs=bcs)
    Q = O.quadrature(q)
    f0 = np.empty((Q["Q"], NY, NX))
    for y in range(NY):
        for x in range(NX):
            f0[:, y, x] = O.equilibrium(q, 1.0, (u0[0, y, x], u0[1, y, x]))
    p = O.poiseuille_struct(1.0, 0.05, 0.1, NX, NY, 1.0, (1.0, 1.0), 0.0)
    f = O.run(q, p, O.collision("TRT", list(taus), force=False), bcs, f0, 0, STEPS - 1)
    cx, cy = np.array(Q["cx"], dtype=float), np.array(Q["cy"], dtype=float)
    rho = f.sum(axis=0)
    ref = float(np.sum((np.tensordot(cx, f, 1) / rho - ut[0]) ** 2 + (np.tensordot(cy, f, 1) / rho - ut[1]) ** 2))
    assert L == pytest.approx(ref, rel=1e-13)


@pytest.mark.parametrize("kind", ["TRT", "MRT"])
def test_walled_tangents_match_central_differences(lbm, O, kind):
    u0, ut = _fields(lbm)
    q, taus, F = "D2Q9", [0.8, 1.1], [2e-6, 0.0]
    bcs = _walls(O)
    v = np.random.default_rng(6).normal(size=u0.shape)

    def value(dt0=0.0, dt1=0.0, dfx=0.0, du=0.0):
        return O.tangent_loss(q, kind, (taus[0] + dt0, taus[1] + dt1), (F[0] + dfx, F[1]), u0 + du * v, ut, STEPS,
                              bcs=bcs)[0]

    def fd(fun, h):
        return (fun(-2 * h) - 8 * fun(-h) + 8 * fun(h) - fun(2 * h)) / (12 * h)

    for seed, du0, ref in [((1, 0, 0, 0), None, fd(lambda e: value(dt0=e), 1e-4)),
                           ((0, 1, 0, 0), None, fd(lambda e: value(dt1=e), 1e-4)),
                           ((0, 0, 1, 0), None, fd(lambda e: value(dfx=e), 1e-7)),
                           ((0, 0, 0, 0), v, fd(lambda e: value(du=e), 1e-5))]:
        _, d = O.tangent_loss(q, kind, taus, F, u0, ut, STEPS, seed=seed, du0=du0, bcs=bcs)
        assert d == pytest.approx(ref, rel=1e-6, abs=1e-13), (seed, d, ref)
