"""The reference's own known-answer tests (test/*.jl), run through the CUDA path."""
import numpy as np
import pytest

from gpu_cases import QUADS

pytestmark = pytest.mark.gpu


def _torch():
    import torch
    return torch


@pytest.mark.parametrize("qname", QUADS)
def test_srt_tau1_returns_equilibrium(lbm_gpu, qname):
    """test/quadrature.jl:64-96: one SRT(1.0) collision of an equilibrium node returns it."""
    lbm = lbm_gpu
    torch = _torch()
    q = lbm.Quadratures[qname]
    f = lbm.equilibrium(q, 1.0, (0.1, 0.1), 1.0).reshape(q.Q, 1, 1)
    f_in = torch.tensor(f, device="cuda")
    f_out = torch.empty_like(f_in)
    lbm.collide(lbm.SRT(1.0), q, f_in, f_out)
    assert np.allclose(f_out.cpu().numpy(), f, atol=1e-4)


@pytest.mark.parametrize("qname", QUADS)
def test_stream_and_collide_keep_equilibrium(lbm_gpu, qname):
    """test/quadrature.jl:98-121: four SRT(1) collide + stream steps on a 1 x 1 lattice."""
    lbm = lbm_gpu
    torch = _torch()
    q = lbm.Quadratures[qname]
    f = lbm.equilibrium(q, 1.0, (0.1, 0.1), 1.0).reshape(q.Q, 1, 1)
    f_inn = torch.tensor(f, device="cuda")
    f_out = torch.empty_like(f_inn)
    for _ in range(4):
        lbm.collide(lbm.SRT(1.0), q, f_inn, f_out)
        lbm.stream(q, f_out, f_inn)
    assert np.allclose(f_inn.cpu().numpy(), f, atol=1e-5)


@pytest.mark.parametrize("qname", QUADS)
def test_multispeed_periodic_stream(lbm_gpu, qname):
    """test/quadrature.jl:132-147: streaming a 1 x 1 lattice with |c| up to 3 is the identity."""
    lbm = lbm_gpu
    torch = _torch()
    q = lbm.Quadratures[qname]
    f = lbm.equilibrium(q, 1.0, (0.0, 0.0), 1.0).reshape(q.Q, 1, 1)
    f_in = torch.tensor(f, device="cuda")
    f_new = torch.empty_like(f_in)
    lbm.stream(q, f_in, f_new)
    assert np.allclose(f_new.cpu().numpy(), f)


def test_trt_equal_taus_is_srt(lbm_gpu):
    """test/collision_models.jl:3-55: TRT(τ, τ) ≡ SRT(τ) for one collision on 10 x 10 and for
    10-step Poiseuille runs over τ ∈ {0.51 ... 1.1}."""
    lbm = lbm_gpu
    torch = _torch()
    q = lbm.D2Q9()
    f = np.ascontiguousarray(np.broadcast_to(q.weights[:, None, None], (9, 10, 10)))
    f_in = torch.tensor(f, device="cuda")
    a, b = torch.empty_like(f_in), torch.empty_like(f_in)
    lbm.collide(lbm.SRT(0.8), q, f_in, a)
    lbm.collide(lbm.TRT(0.8, 0.8), q, f_in, b)
    assert np.allclose(a.cpu().numpy(), b.cpu().numpy(), rtol=1.5e-8)
    for tau in [0.51, 0.6, 0.7, 0.8, 0.9, 1.0, 1.1]:
        nu = (tau - 0.5) / q.speed_of_sound_squared
        problem = lbm.PoiseuilleFlow(nu, 1, static=False)
        res = []
        for cm in (lbm.SRT(tau), lbm.TRT(tau, tau)):
            pm = lbm.ProcessingMethod(problem, False, 10)
            m = lbm.LatticeBoltzmannModel(problem, q, collision_model=cm, process_method=pm)
            lbm.simulate(m, time=range(0, 11))
            res.append(m.f_stream)
            m.close()
        assert np.allclose(res[0], res[1], rtol=1.5e-8)


def test_mrt_tau1_is_srt(lbm_gpu):
    """test/collision_models.jl:57-114: MRT(q, τ) ≡ SRT(τ) at τ = 1 (the reference marks the
    other τ as broken: the regularisation differs by design)."""
    lbm = lbm_gpu
    q = lbm.D2Q9()
    problem = lbm.PoiseuilleFlow((1.0 - 0.5) / 3.0, 1, static=False)
    res = []
    for cm in (lbm.SRT(1.0), lbm.MRT(q, 1.0)):
        pm = lbm.ProcessingMethod(problem, False, 10)
        m = lbm.LatticeBoltzmannModel(problem, q, collision_model=cm, process_method=pm)
        lbm.simulate(m, time=range(0, 11))
        res.append(m.f_stream)
        m.close()
    assert np.allclose(res[0], res[1], rtol=1.5e-8)


def test_bounce_back_operator_matches_oracle(lbm_gpu, O):
    """apply!(bcs, q, f_new, f_old) on device arrays against the oracle, all four walls."""
    lbm = lbm_gpu
    torch = _torch()
    q = lbm.D2Q9()
    rng = np.random.default_rng(5)
    f_new = rng.random((9, 6, 7))
    f_old = rng.random((9, 6, 7))
    bcs = [lbm.BounceBack(lbm.East(), (1, 7), (1, 6)), lbm.BounceBack(lbm.South(), (1, 7), (1, 6)),
           lbm.BounceBack(lbm.West(), (1, 7), (1, 6)), lbm.MovingWall(lbm.North(), (1, 7), (1, 6), [0.01, 0.0])]
    obcs = [O.bc("bounce_back", "east", (1, 7), (1, 6)), O.bc("bounce_back", "south", (1, 7), (1, 6)),
            O.bc("bounce_back", "west", (1, 7), (1, 6)), O.bc("moving_wall", "north", (1, 7), (1, 6), u=(0.01, 0.0))]
    t_new = torch.tensor(f_new, device="cuda")
    t_old = torch.tensor(f_old, device="cuda")
    lbm.apply(bcs, q, t_new, t_old)
    ref = O.apply_bcs("D2Q9", obcs, f_new, f_old)
    np.testing.assert_allclose(t_new.cpu().numpy(), ref, rtol=1e-15)
