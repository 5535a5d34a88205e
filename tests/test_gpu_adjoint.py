"""Adjoint gradients (lbm_adjoint_*) against central finite differences of the device forward
model (FP64) and of the oracle's CPU restatement of the reference loop."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NX = NY = 32
STEPS = 120


def _setup(lbm, storage="f64", nsteps=STEPS, tau_s=0.8, F=(2e-6, -1e-6), slots=0, bcs=()):
    q = lbm.D2Q9()
    tau_a = lbm.trt_magic(tau_s)
    return lbm.AdjointProblem(q, NX, NY, lbm.TRT.fields(tau_s, tau_a), force=F, nsteps=nsteps,
                              slots=slots, storage=storage, boundary_conditions=bcs)


def _fields(lbm):
    u0 = lbm.divergence_free_field(NX, NY, kmax=4, amplitude=0.01, seed=1)
    ut = lbm.divergence_free_field(NX, NY, kmax=4, amplitude=0.01, seed=2)
    return u0, ut


def _loss(lbm, u0, ut, tau_s, tau_a, F, storage="f64"):
    q = lbm.D2Q9()
    p = lbm.AdjointProblem(q, NX, NY, lbm.TRT.fields(tau_s, tau_a), force=F, nsteps=STEPS, storage=storage)
    L = p.loss(u0, ut)
    p.close()
    return L


def test_adjoint_matches_finite_differences(lbm_gpu):
    lbm = lbm_gpu
    u0, ut = _fields(lbm)
    tau_s, F = 0.8, (2e-6, -1e-6)
    tau_a = lbm.trt_magic(tau_s)
    prob = _setup(lbm, tau_s=tau_s, F=F)
    res = prob.run(u0, ut)
    prob.close()
    # fourth-order central differences: the loss is ~0.2, so a two-point difference with a step
    # of 1e-6 carries a rounding error of ~1e-11, the size of the smallest gradients checked here
    def fd(fun, h):
        return (fun(-2 * h) - 8 * fun(-h) + 8 * fun(h) - fun(2 * h)) / (12 * h)

    fd_ts = fd(lambda e: _loss(lbm, u0, ut, tau_s + e, tau_a, F), 1e-4)
    fd_ta = fd(lambda e: _loss(lbm, u0, ut, tau_s, tau_a + e, F), 1e-4)
    fd_fx = fd(lambda e: _loss(lbm, u0, ut, tau_s, tau_a, (F[0] + e, F[1])), 1e-7)
    rng = np.random.default_rng(7)
    v = rng.normal(size=u0.shape)
    fd_u = fd(lambda e: _loss(lbm, u0 + e * v, ut, tau_s, tau_a, F), 1e-5)
    for ad, fd in [(res["dtau_s"], fd_ts), (res["dtau_a"], fd_ta), (res["dF"][0], fd_fx),
                   (float(np.sum(res["grad_u0"] * v)), fd_u)]:
        assert abs(ad - fd) <= 1e-6 * max(abs(fd), 1e-12), (ad, fd)


def test_adjoint_matches_oracle_finite_differences(lbm_gpu, O):
    """The same loss evaluated with the oracle's collide -> stream loop (the CPU restatement of
    the reference) gives the same value and central differences as the adjoint."""
    lbm = lbm_gpu
    u0, ut = _fields(lbm)
    tau_s, F = 0.8, (2e-6, -1e-6)
    tau_a = lbm.trt_magic(tau_s)

    def oracle_loss(ts, ta, u):
        p = O.poiseuille_struct(1.0, 0.05, 0.1, NX, NY, 1.0, (1.0, 1.0), 1.0)
        sc = O.problem_scalars(p)
        p.G = F[0] / (p.u_max * sc["delta_t"] * sc["viscosity"])
        f0 = np.empty((9, NY, NX))
        for y in range(NY):
            for x in range(NX):
                f0[:, y, x] = O.equilibrium("D2Q9", 1.0, (u[0, y, x], u[1, y, x]))
        f = O.run("D2Q9", p, O.collision("TRT", [ts, ta], force=True), [], f0, 0, STEPS - 1, dt=sc["delta_t"])
        rho = f.sum(axis=0)
        cx = np.array([0, -1, -1, -1, 0, 1, 1, 1, 0])
        cy = np.array([0, 1, 0, -1, -1, -1, 0, 1, 1])
        ux = np.tensordot(cx, f, 1) / rho
        uy = np.tensordot(cy, f, 1) / rho
        return float(np.sum((ux - ut[0]) ** 2 + (uy - ut[1]) ** 2))

    Fx_only = (F[0], 0.0)  # the oracle's Poiseuille force is along x
    prob = _setup(lbm, tau_s=tau_s, F=Fx_only)
    res = prob.run(u0, ut)
    prob.close()
    assert res["loss"] == pytest.approx(oracle_loss(tau_s, tau_a, u0), rel=1e-10)
    h = 1e-6
    fd_ts = (oracle_loss(tau_s + h, tau_a, u0) - oracle_loss(tau_s - h, tau_a, u0)) / (2 * h)
    assert abs(res["dtau_s"] - fd_ts) <= 1e-6 * abs(fd_ts)
    rng = np.random.default_rng(3)
    v = rng.normal(size=u0.shape)
    fd_u = (oracle_loss(tau_s, tau_a, u0 + h * v) - oracle_loss(tau_s, tau_a, u0 - h * v)) / (2 * h)
    assert abs(float(np.sum(res["grad_u0"] * v)) - fd_u) <= 1e-6 * abs(fd_u)


@pytest.mark.parametrize("kind", ["TRT", "SRT"])
def test_adjoint_matches_oracle_forward_mode(lbm_gpu, O, kind):
    """At 64 x 64: the adjoint's ∂L/∂τ_s, ∂L/∂τ_a, ∂L/∂F and a directional ∂L/∂u0 against the
    forward-mode derivatives of the oracle's loop (dual numbers through its collide / stream;
    the stand-in for ForwardDiff through the reference)."""
    lbm = lbm_gpu
    n, steps = 64, 200
    u0 = lbm.divergence_free_field(n, n, kmax=8, amplitude=0.01, seed=21)
    ut = lbm.divergence_free_field(n, n, kmax=8, amplitude=0.01, seed=22)
    tau_s, F = 0.8, (2e-6, -1e-6)
    tau_a = lbm.trt_magic(tau_s) if kind == "TRT" else tau_s
    cm = lbm.TRT.fields(tau_s, tau_a) if kind == "TRT" else lbm.SRT(tau_s)
    p = lbm.AdjointProblem(lbm.D2Q9(), n, n, cm, force=F, nsteps=steps)
    res = p.run(u0, ut)
    p.close()
    v = np.random.default_rng(9).normal(size=u0.shape)
    nt = O.max_threads()

    def tangent(seed, du0=None):
        return O.tangent_loss("D2Q9", kind, (tau_s, tau_a), F, u0, ut, steps, seed=seed, du0=du0, nthreads=nt)

    L, d_ts = tangent((1, 0, 0, 0))
    assert res["loss"] == pytest.approx(L, rel=1e-10)
    pairs = [(res["dtau_s"], d_ts), (res["dF"][0], tangent((0, 0, 1, 0))[1]),
             (res["dF"][1], tangent((0, 0, 0, 1))[1]),
             (float(np.sum(res["grad_u0"] * v)), tangent((0, 0, 0, 0), v)[1])]
    if kind == "TRT":
        pairs.append((res["dtau_a"], tangent((0, 1, 0, 0))[1]))
    for ad, fm in pairs:
        assert ad == pytest.approx(fm, rel=1e-8), (ad, fm)


@pytest.mark.parametrize("walls", [False, True])
def test_checkpoint_slots_do_not_change_gradients(lbm_gpu, walls):
    """Binomial checkpointing with 1, 2, 5, the default and T - 1 slots: the same forward states are
    recomputed, so loss and gradients are bitwise the same; fewer slots cost more forward steps, and
    with s slots no step is recomputed more than r times, C(s + r, s) >= T."""
    lbm = lbm_gpu
    u0, ut = _fields(lbm)
    bcs = _walls(lbm) if walls else ()
    outs, infos = [], []
    for sl in (1, 2, 5, 0, STEPS - 1):
        prob = _setup(lbm, slots=sl, bcs=bcs)
        outs.append(prob.run(u0, ut))
        infos.append(prob.info())
        prob.close()
    for o in outs[1:]:
        assert o["loss"] == outs[0]["loss"]
        np.testing.assert_array_equal(o["grad_u0"], outs[0]["grad_u0"])
        assert o["dtau_s"] == outs[0]["dtau_s"]
    from math import comb
    for info in infos:
        s = info["slots"]
        r = next(r for r in range(1, STEPS + 1) if comb(s + r, s) >= STEPS)
        assert STEPS <= info["forward_steps"] <= (r + 1) * STEPS, info
    assert infos[-1]["forward_steps"] < infos[0]["forward_steps"]
    assert infos[-1]["device_bytes"] > infos[0]["device_bytes"]


def test_fp32_adjoint_close_to_fp64(lbm_gpu):
    lbm = lbm_gpu
    u0, ut = _fields(lbm)
    r = {}
    for st in ("f64", "f32dev"):
        prob = _setup(lbm, storage=st)
        r[st] = prob.run(u0, ut)
        prob.close()
    assert r["f32dev"]["loss"] == pytest.approx(r["f64"]["loss"], rel=1e-4)
    g64, g32 = r["f64"]["grad_u0"], r["f32dev"]["grad_u0"]
    assert np.max(np.abs(g32 - g64)) <= 1e-3 * np.max(np.abs(g64))


def test_autograd_function_returns_the_adjoint_gradients(lbm_gpu):
    """LBMLoss (the torch.autograd counterpart of a ChainRulesCore.rrule for this loss): its
    backward gives the adjoint's ∂L/∂u0, the total ∂L/∂τ_s along the magic relation and ∂L/∂F,
    and a gradient step on u0 lowers the loss."""
    torch = pytest.importorskip("torch")
    lbm = lbm_gpu
    u0, ut = _fields(lbm)
    q = lbm.D2Q9()

    def factory(tau, F):
        return lbm.AdjointProblem(q, NX, NY, lbm.TRT.fields(tau, lbm.trt_magic(tau)), force=F, nsteps=STEPS)

    u = torch.tensor(u0, dtype=torch.float64, requires_grad=True)
    tau = torch.tensor(0.8, dtype=torch.float64, requires_grad=True)
    F = torch.tensor([2e-6, -1e-6], dtype=torch.float64, requires_grad=True)
    loss = lbm.LBMLoss.apply(u, tau, F, factory, ut)
    loss.backward()
    prob = factory(0.8, (2e-6, -1e-6))
    ref = prob.run(u0, ut)
    prob.close()
    assert float(loss.detach()) == ref["loss"]
    np.testing.assert_array_equal(u.grad.numpy(), ref["grad_u0"])
    assert float(tau.grad) == pytest.approx(lbm.magic_total_derivative(ref, 0.8), rel=1e-12)
    np.testing.assert_allclose(F.grad.numpy(), np.asarray(ref["dF"]), rtol=1e-12)
    with torch.no_grad():
        u_step = u - 1e-3 * u.grad / u.grad.abs().max()
    assert float(lbm.LBMLoss.apply(u_step, tau, F, factory, ut).detach()) < float(loss.detach())


@pytest.mark.parametrize("qname,coll", [("D2Q13", "TRT"), ("D2Q9", "SRT"), ("D2Q13", "SRT")])
def test_other_sets_and_srt_match_finite_differences(lbm_gpu, qname, coll):
    """The adjoint of D2Q13 and of SRT (one relaxation time): ∂L/∂τ and ∂L/∂F_x against
    fourth-order central differences of the device forward model."""
    lbm = lbm_gpu
    q = lbm.Quadratures[qname]
    n, steps = 24, 60
    u0 = lbm.divergence_free_field(n, n, kmax=3, amplitude=0.01, seed=3)
    ut = lbm.divergence_free_field(n, n, kmax=3, amplitude=0.01, seed=4)

    def cm(tau):
        return lbm.SRT(tau) if coll == "SRT" else lbm.TRT.fields(tau, 1.1)

    def loss(tau, F):
        p = lbm.AdjointProblem(q, n, n, cm(tau), force=F, nsteps=steps)
        L = p.loss(u0, ut)
        p.close()
        return L

    def fd(fun, h):
        return (fun(-2 * h) - 8 * fun(-h) + 8 * fun(h) - fun(2 * h)) / (12 * h)

    tau, F = 0.85, (3e-6, 1e-6)
    p = lbm.AdjointProblem(q, n, n, cm(tau), force=F, nsteps=steps)
    res = p.run(u0, ut)
    p.close()
    fd_tau = fd(lambda e: loss(tau + e, F), 1e-4)
    fd_fx = fd(lambda e: loss(tau, (F[0] + e, F[1])), 1e-7)
    assert res["dtau_s"] == pytest.approx(fd_tau, rel=1e-6, abs=1e-12)
    assert res["dF"][0] == pytest.approx(fd_fx, rel=1e-6, abs=1e-12)


def _walls(lbm, nx=NX, ny=NY, lid=False):
    if lid:
        return [lbm.BounceBack(lbm.East(), (1, nx), (1, ny)), lbm.BounceBack(lbm.South(), (1, nx), (1, ny)),
                lbm.BounceBack(lbm.West(), (1, nx), (1, ny)), lbm.MovingWall(lbm.North(), (1, nx), (1, ny), (0.01, 0.0))]
    return [lbm.BounceBack(lbm.North(), (1, nx), (1, ny)), lbm.BounceBack(lbm.South(), (1, nx), (1, ny))]


def _owalls(O, nx=NX, ny=NY, lid=False):
    if lid:
        return [O.bc("bounce_back", "east", (1, nx), (1, ny)), O.bc("bounce_back", "south", (1, nx), (1, ny)),
                O.bc("bounce_back", "west", (1, nx), (1, ny)),
                O.bc("moving_wall", "north", (1, nx), (1, ny), u=(0.01, 0.0))]
    return [O.bc("bounce_back", "north", (1, nx), (1, ny)), O.bc("bounce_back", "south", (1, nx), (1, ny))]


def test_walled_channel_adjoint_matches_finite_differences(lbm_gpu):
    """The 32 x 32 TRT channel with bounce-back walls North and South and a body force (the
    benchmark channel's boundaries, bounce_back.jl:8-72): ∂L/∂τ_s, ∂L/∂τ_a, ∂L/∂F_x and a
    directional ∂L/∂u0 against fourth-order central differences of the device forward model."""
    lbm = lbm_gpu
    u0, ut = _fields(lbm)
    tau_s, F = 0.8, (2e-6, 0.0)
    tau_a = lbm.trt_magic(tau_s)
    bcs = _walls(lbm)
    prob = _setup(lbm, tau_s=tau_s, F=F, bcs=bcs, slots=6)
    res = prob.run(u0, ut)
    prob.close()

    def loss(ts, ta, Fx, u):
        p = lbm.AdjointProblem(lbm.D2Q9(), NX, NY, lbm.TRT.fields(ts, ta), force=(Fx, 0.0), nsteps=STEPS,
                               boundary_conditions=_walls(lbm))
        L = p.loss(u, ut)
        p.close()
        return L

    def fd(fun, h):
        return (fun(-2 * h) - 8 * fun(-h) + 8 * fun(h) - fun(2 * h)) / (12 * h)

    v = np.random.default_rng(17).normal(size=u0.shape)
    checks = [(res["dtau_s"], fd(lambda e: loss(tau_s + e, tau_a, F[0], u0), 1e-4)),
              (res["dtau_a"], fd(lambda e: loss(tau_s, tau_a + e, F[0], u0), 1e-4)),
              (res["dF"][0], fd(lambda e: loss(tau_s, tau_a, F[0] + e, u0), 1e-7)),
              (float(np.sum(res["grad_u0"] * v)), fd(lambda e: loss(tau_s, tau_a, F[0], u0 + e * v), 1e-5))]
    for ad, ref in checks:
        assert abs(ad - ref) <= 1e-6 * max(abs(ref), 1e-12), (ad, ref)


@pytest.mark.parametrize("lid", [False, True])
def test_walled_adjoint_matches_oracle_forward_mode(lbm_gpu, O, lid):
    """Walled channel, and a lid-driven cavity (bounce-back East, South, West, moving lid North):
    the adjoint's derivatives against the forward-mode (dual-number) derivatives of the oracle's
    collide -> stream -> apply! loop with the same boundary list (≤ 1e-8)."""
    lbm = lbm_gpu
    u0, ut = _fields(lbm)
    tau_s, F = 0.8, (2e-6, 0.0)
    tau_a = lbm.trt_magic(tau_s)
    prob = _setup(lbm, tau_s=tau_s, F=F, bcs=_walls(lbm, lid=lid), slots=4)
    res = prob.run(u0, ut)
    prob.close()
    v = np.random.default_rng(19).normal(size=u0.shape)
    obcs = _owalls(O, lid=lid)

    def tangent(seed, du0=None):
        return O.tangent_loss("D2Q9", "TRT", (tau_s, tau_a), F, u0, ut, STEPS, seed=seed, du0=du0, bcs=obcs)

    L, d_ts = tangent((1, 0, 0, 0))
    assert res["loss"] == pytest.approx(L, rel=1e-10)
    for ad, fm in [(res["dtau_s"], d_ts), (res["dtau_a"], tangent((0, 1, 0, 0))[1]),
                   (res["dF"][0], tangent((0, 0, 1, 0))[1]),
                   (float(np.sum(res["grad_u0"] * v)), tangent((0, 0, 0, 0), v)[1])]:
        assert ad == pytest.approx(fm, rel=1e-8), (ad, fm)


@pytest.mark.parametrize("qname,bc", [("D2Q9", "none"), ("D2Q9", "walls"), ("D2Q9", "lid"), ("D2Q13", "none")])
def test_mrt_adjoint_matches_oracle_forward_mode(lbm_gpu, O, qname, bc):
    """Regularised MRT (mrt.jl:56-118; a second-order set relaxes its second-order Hermite
    coefficient with τ_2, which also scales the force shift): the adjoint's ∂L/∂τ_2, ∂L/∂F and a
    directional ∂L/∂u0 against the forward-mode derivatives of the oracle's loop, periodic, with
    channel walls and as a lid-driven cavity (≤ 1e-8)."""
    lbm = lbm_gpu
    q = lbm.Quadratures[qname]
    u0, ut = _fields(lbm)
    tau, F = 0.8, (2e-6, -1e-6) if bc == "none" else (2e-6, 0.0)
    bcs = () if bc == "none" else _walls(lbm, lid=(bc == "lid"))
    obcs = () if bc == "none" else _owalls(O, lid=(bc == "lid"))
    prob = lbm.AdjointProblem(q, NX, NY, lbm.MRT(q, tau), force=F, nsteps=STEPS, slots=5,
                              boundary_conditions=bcs)
    res = prob.run(u0, ut)
    prob.close()
    v = np.random.default_rng(23).normal(size=u0.shape)

    def tangent(seed, du0=None):
        return O.tangent_loss(qname, "MRT", (tau, tau), F, u0, ut, STEPS, seed=seed, du0=du0, bcs=obcs,
                              nthreads=O.max_threads())

    L, d_tau = tangent((0, 1, 0, 0))
    assert res["loss"] == pytest.approx(L, rel=1e-10)
    assert tangent((1, 0, 0, 0))[1] == 0.0  # the first-order relaxation time never reaches the outputs
    pairs = [(res["dtau_s"], d_tau), (res["dF"][0], tangent((0, 0, 1, 0))[1]),
             (float(np.sum(res["grad_u0"] * v)), tangent((0, 0, 0, 0), v)[1])]
    if bc == "none":
        pairs.append((res["dF"][1], tangent((0, 0, 0, 1))[1]))
    assert res["dtau_a"] == 0.0
    for ad, fm in pairs:
        assert ad == pytest.approx(fm, rel=1e-8), (ad, fm)


def test_mrt_adjoint_matches_finite_differences(lbm_gpu):
    """∂L/∂τ, ∂L/∂F_x and a directional ∂L/∂u0 of the MRT channel with walls against fourth-order
    central differences of the device forward model (FP64)."""
    lbm = lbm_gpu
    q = lbm.D2Q9()
    u0, ut = _fields(lbm)
    tau, Fx = 0.8, 2e-6

    def loss(t, fx, u):
        p = lbm.AdjointProblem(q, NX, NY, lbm.MRT(q, t), force=(fx, 0.0), nsteps=STEPS,
                               boundary_conditions=_walls(lbm))
        L = p.loss(u, ut)
        p.close()
        return L

    def fd(fun, h):
        return (fun(-2 * h) - 8 * fun(-h) + 8 * fun(h) - fun(2 * h)) / (12 * h)

    prob = lbm.AdjointProblem(q, NX, NY, lbm.MRT(q, tau), force=(Fx, 0.0), nsteps=STEPS,
                              boundary_conditions=_walls(lbm))
    res = prob.run(u0, ut)
    prob.close()
    v = np.random.default_rng(29).normal(size=u0.shape)
    for ad, ref in [(res["dtau_s"], fd(lambda e: loss(tau + e, Fx, u0), 1e-4)),
                    (res["dF"][0], fd(lambda e: loss(tau, Fx + e, u0), 1e-7)),
                    (float(np.sum(res["grad_u0"] * v)), fd(lambda e: loss(tau, Fx, u0 + e * v), 1e-5))]:
        assert abs(ad - ref) <= 1e-6 * max(abs(ref), 1e-12), (ad, ref)


def test_mrt_fp32_adjoint_close_to_fp64(lbm_gpu):
    lbm = lbm_gpu
    q = lbm.D2Q9()
    u0, ut = _fields(lbm)
    r = {}
    for st in ("f64", "f32dev"):
        prob = lbm.AdjointProblem(q, NX, NY, lbm.MRT(q, 0.8), force=(2e-6, -1e-6), nsteps=STEPS, storage=st)
        r[st] = prob.run(u0, ut)
        prob.close()
    assert r["f32dev"]["loss"] == pytest.approx(r["f64"]["loss"], rel=1e-4)
    assert r["f32dev"]["dtau_s"] == pytest.approx(r["f64"]["dtau_s"], rel=1e-3)
    g64, g32 = r["f64"]["grad_u0"], r["f32dev"]["grad_u0"]
    assert np.max(np.abs(g32 - g64)) <= 1e-3 * np.max(np.abs(g64))
