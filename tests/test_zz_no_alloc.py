"""lbm_reduce_noalloc: the reductions for callers that cannot allocate device memory, called
through the C ABI and checked against the context-based lbm_reduce on the same populations,
twice in a row (the second call reuses the shared static scratch array).

This file is collected last on purpose: it exercises the one entry point that keeps state in
a file-scope device array, after every other test has run (and it also passes alone)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _fn(lbm):
    L = lbm._native.lib()
    fn = L.lbm_reduce_noalloc
    fn.argtypes = [C.c_int32, C.POINTER(C.c_double), C.c_double, C.c_int64, C.c_int64, C.c_void_p, C.c_int32,
                   C.POINTER(lbm._native.LbmAnalytic), C.c_void_p, C.c_void_p]
    fn.restype = C.c_int32
    return fn


def test_no_alloc_reduce_matches_context_reduce(lbm_gpu):
    import torch
    lbm = lbm_gpu
    N = lbm._native
    fn = _fn(lbm)
    q = lbm.D2Q9()
    problem = lbm.TaylorGreenVortex(0.1, 1, 96, 80, static=False)
    m = lbm.LatticeBoltzmannModel(problem, q, collision_model=lbm.SRT,
                                  initialization_strategy=lbm.AnalyticalEquilibriumAndOffEquilibrium())
    lbm.run_steps(m, 0, 49)
    t = 50
    fields = lbm.analytic_fields(q, problem, t * problem.delta_t())
    tau = q.speed_of_sound_squared * problem.lattice_viscosity()
    _, _, xs, ys = lbm.problem_range(problem)
    expected = {
        N.REDUCE_TRACK_ERRORS: m.lattice.reduce(N.REDUCE_TRACK_ERRORS, fields, tau=tau, u_max=problem.u_max),
        N.REDUCE_COMPARE: m.lattice.reduce(N.REDUCE_COMPARE, fields, u_max=problem.u_max, area=xs * ys),
        N.REDUCE_MEAN_VELOCITY: m.lattice.reduce(N.REDUCE_MEAN_VELOCITY),
        N.REDUCE_CONSERVED: m.lattice.reduce(N.REDUCE_CONSERVED),
    }
    f_dev = torch.tensor(m.f_stream, device="cuda")
    dev_fields = {k: torch.tensor(v, device="cuda") for k, v in fields.items()}
    m.close()
    an = N.LbmAnalytic()
    for name, tensor in dev_fields.items():
        setattr(an, name, C.cast(C.c_void_p(tensor.data_ptr()), N._DP))
    an.on_device = 1
    weights = np.ascontiguousarray(q.weights)
    wptr = weights.ctypes.data_as(C.POINTER(C.c_double))
    out = torch.zeros(16, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    for call in range(2):
        for kind, ref in expected.items():
            an.tau = tau if kind == N.REDUCE_TRACK_ERRORS else 0.0
            an.u_max = problem.u_max
            an.area = xs * ys if kind == N.REDUCE_COMPARE else 0.0
            out.fill_(float("nan"))
            st = fn(q.qid, wptr, q.speed_of_sound_squared, 96, 80, f_dev.data_ptr(), kind, C.byref(an),
                    out.data_ptr(), stream.cuda_stream)
            assert st == N.LBM_OK, (call, kind, st)
            torch.cuda.synchronize()
            got = out.cpu().numpy()[: len(ref)]
            np.testing.assert_allclose(got, ref, rtol=TOL, atol=1e-300, err_msg=f"call {call} kind {kind}")


def test_no_alloc_reduce_rejects_oversized_lattices(lbm_gpu):
    """Lattices of 2^31 nodes or more are refused before any device work."""
    lbm = lbm_gpu
    fn = _fn(lbm)
    w = np.ascontiguousarray(lbm.D2Q9().weights)
    st = fn(2, w.ctypes.data_as(C.POINTER(C.c_double)), 3.0, 1 << 16, 1 << 15, 1, lbm._native.REDUCE_CONSERVED,
            None, 1, None)
    assert st == lbm._native.LBM_ERR_INVALID
