"""The reference's own known-answer tests (test/runtests.jl, test/quadrature.jl,
test/collision_models.jl, test/initial_conditions.jl) applied to the oracle, which pins it
to the reference's algorithm beyond the printed notebook rows."""
import math

import numpy as np
import pytest

QUADS = ["D2Q4", "D2Q5", "D2Q9", "D2Q13", "D2Q17", "D2Q21", "D2Q37"]


def _hermite_sum(O, q, n):
    Q = O.quadrature(q)
    tot = None
    for i in range(Q["Q"]):
        h = Q["w"][i] * O.hermite(q, n, (Q["cx"][i], Q["cy"][i]))
        tot = h if tot is None else tot + h
    return tot


@pytest.mark.parametrize("q", QUADS)
def test_symmetry(O, q):
    """test/quadrature.jl:1-19: Σw = 1 and Σ w H_n(c) = 0 for n ≤ order ÷ 2."""
    Q = O.quadrature(q)
    assert sum(Q["w"]) == pytest.approx(1.0)
    for n in range(1, Q["order"] // 2 + 1):
        assert np.all(np.abs(_hermite_sum(O, q, n)) <= 1e-15)


@pytest.mark.parametrize("q", QUADS)
def test_opposite(O, q):
    """test/quadrature.jl:124-130."""
    Q = O.quadrature(q)
    for i in range(Q["Q"]):
        o = Q["opposite"][i]
        assert Q["cx"][i] + Q["cx"][o] == 0 and Q["cy"][i] + Q["cy"][o] == 0


@pytest.mark.parametrize("q", QUADS)
def test_equilibrium_moments(O, q):
    """test/quadrature.jl:21-62: ρ, u and T recovered from equilibrium(q, ρ, u, T)."""
    for u in ([0.001, 0.001], [0.1, 0.1]):
        f = O.hermite_equilibrium(q, 1.0, u, 1.0)
        m = O.moments(q, f)
        assert m[0] == pytest.approx(1.0)
        assert m[1] == pytest.approx(u[0]) and m[2] == pytest.approx(u[1])
        if u[0] == 0.001:
            assert m[4] == pytest.approx(1.0, abs=1e-5)
    f = O.hermite_equilibrium(q, 1.0, [0.0, 0.0], 1.0)
    assert O.moments(q, f)[4] == pytest.approx(1.0)


@pytest.mark.parametrize("q", QUADS)
def test_equilibrium_density_momentum_logspace(O, q):
    """test/runtests.jl:56-118: collision equilibrium ρ / momentum for u ∈ logspace(2, -9, 12)."""
    for u in 10.0 ** np.linspace(2, -9, 12):
        for v in ([0, 0], [u, 0.0], [0.0, u], [u, u]):
            f = O.equilibrium(q, 1.0, v)
            if not math.isclose(f.sum(), 1.0, rel_tol=1e-10, abs_tol=1e-8):
                f = O.hermite_equilibrium(q, 1.0, v, 1.0)  # as the reference's test helper does
            m = O.moments(q, f)
            assert m[0] == pytest.approx(1.0, rel=1e-10, abs=1e-8)
            assert m[1] == pytest.approx(v[0], abs=1e-11, rel=1e-6)
            assert m[2] == pytest.approx(v[1], abs=1e-11, rel=1e-6)


@pytest.mark.parametrize("q", QUADS)
def test_srt_tau1_and_stream_collide(O, q):
    """test/quadrature.jl:64-121."""
    Q = O.quadrature(q)["Q"]
    f = O.hermite_equilibrium(q, 1.0, [0.1, 0.1], 1.0).reshape(Q, 1, 1)
    out = O.collide(q, f, O.collision("SRT", [1.0]))
    assert np.allclose(out, f, atol=1e-4)
    g = f.copy()
    for _ in range(4):
        g = O.stream(q, O.collide(q, g, O.collision("SRT", [1.0])))
    assert np.allclose(g, f, atol=1e-5)
    z = O.hermite_equilibrium(q, 1.0, [0.0, 0.0], 1.0).reshape(Q, 1, 1)
    assert np.allclose(O.stream(q, z), z)


def test_hermite_values(O):
    """test/runtests.jl:17-51 (with cs = 1/3 scaling the isotropic terms for D2Q9)."""
    H2 = O.hermite("D2Q9", 2, (1, 0))
    assert np.allclose(H2, [1 - 1 / 3, 0, 0, -1 / 3])
    H1 = O.hermite("D2Q9", 1, (1, 0))
    assert np.allclose(H1, [1, 0])


def test_trt_equal_taus_is_srt(O):
    """test/collision_models.jl:3-55, on the oracle."""
    W = O.quadrature("D2Q9")["w"]
    f = np.ascontiguousarray(np.broadcast_to(W[:, None, None], (9, 10, 10)))
    a = O.collide("D2Q9", f, O.collision("SRT", [0.8]))
    b = O.collide("D2Q9", f, O.collision("TRT", [0.8, 0.8]))
    assert np.allclose(a, b, rtol=1.5e-8)
    for tau in [0.51, 0.6, 0.7, 0.8, 0.9, 1.0, 1.1]:
        p = O.poiseuille((tau - 0.5) / 3.0, 1)
        bcs = [O.bc("bounce_back", "north", (1, 3), (1, 5)), O.bc("bounce_back", "south", (1, 3), (1, 5))]
        f0 = O.initialize(O.INIT_EQUILIBRIUM, "D2Q9", p)
        ra = O.run("D2Q9", p, O.collision("SRT", [tau]), bcs, f0, 0, 10)
        rb = O.run("D2Q9", p, O.collision("TRT", [tau, tau]), bcs, f0, 0, 10)
        assert np.allclose(ra, rb, rtol=1.5e-8)


def test_mrt_tau1_is_srt(O):
    """test/collision_models.jl:57-114: equal at τ = 1, different otherwise (@test_broken there)."""
    for tau in [0.8, 1.0]:
        p = O.poiseuille((tau - 0.5) / 3.0, 1)
        bcs = [O.bc("bounce_back", "north", (1, 3), (1, 5)), O.bc("bounce_back", "south", (1, 3), (1, 5))]
        f0 = O.initialize(O.INIT_EQUILIBRIUM, "D2Q9", p)
        ra = O.run("D2Q9", p, O.collision("SRT", [tau]), bcs, f0, 0, 10)
        rb = O.run("D2Q9", p, O.collision("MRT", [tau, tau]), bcs, f0, 0, 10)
        assert np.allclose(ra, rb, rtol=1.5e-8) == (tau == 1.0)


def _isapprox(a, b, rtol=math.sqrt(np.finfo(float).eps)):
    """Julia's isapprox for numbers and arrays: norm(a - b) <= rtol * max(norm(a), norm(b))."""
    a, b = np.atleast_1d(np.asarray(a, float)), np.atleast_1d(np.asarray(b, float))
    return np.linalg.norm(a - b) <= rtol * max(np.linalg.norm(a), np.linalg.norm(b))


@pytest.mark.parametrize("q", ["D2Q9", "D2Q13", "D2Q17", "D2Q21"])
def test_initialisation_strategies(O, q):
    """test/initial_conditions.jl:89-214 on InitializationTestProblem(8, ν = 1/cs²), τ = 1."""
    cs = O.quadrature(q)["cs"]
    p = O.init_test_problem(8, 1.0 / cs)
    F = O.problem_fields(p, q, 0.0)
    #            strategy                rho/p ≈ analytic   σ ≈ analytic
    cases = [(O.INIT_CONSTANT_DENSITY, False, False), (O.INIT_EQUILIBRIUM, True, False),
             (O.INIT_VELOCITY_STRESS, False, True), (O.INIT_EQ_OFFEQ, True, True)]
    for strat, rho_ok, sigma_ok in cases:
        f = O.initialize(strat, q, p)
        for y in range(8):
            for x in range(8):
                m = O.moments(q, f[:, y, x], 1.0)
                rho_a, ux_a, uy_a, p_a = F[0, y, x], F[1, y, x], F[2, y, x], F[3, y, x]
                assert _isapprox(m[1:3], [ux_a, uy_a])
                if rho_ok:
                    assert _isapprox(m[0], rho_a) and _isapprox(m[3], p_a)
                elif not _isapprox(rho_a, 1.0):
                    assert not _isapprox(m[0], rho_a) and not _isapprox(m[3], p_a)
                assert _isapprox(m[5:9], F[4:8, y, x]) == sigma_ok
