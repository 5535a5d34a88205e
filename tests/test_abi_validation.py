"""Argument validation of the C ABI: invalid descriptors and handles are rejected with the
documented status before any device work (these calls run without a GPU)."""
import ctypes as C

import numpy as np
import pytest


@pytest.fixture(scope="module")
def L(lbm):
    lbm.build()
    return lbm._native.lib()


def _desc(lbm, qname="D2Q9", nx=8, ny=6, **kw):
    N = lbm._native
    q = lbm.Quadratures[qname]
    d = N.LbmDesc()
    d.quadrature = q.qid
    for i, w in enumerate(q.weights):
        d.weights[i] = float(w)
    d.speed_of_sound_squared = q.speed_of_sound_squared
    d.collision = N.SRT
    d.tau[0] = 0.8
    d.nx, d.ny = nx, ny
    d.storage = N.STORE_F64
    for k, v in kw.items():
        setattr(d, k, v)
    return d


def _create(L, d):
    h = C.c_void_p()
    st = L.lbm_create(C.byref(h), C.byref(d))
    if h.value:
        L.lbm_destroy(h)
    return st


def test_status_strings_and_version(lbm, L):
    N = lbm._native
    assert L.lbm_abi_version() == 1
    for st, text in ((N.LBM_OK, "ok"), (N.LBM_ERR_INVALID, "invalid argument"),
                     (N.LBM_ERR_UNSUPPORTED, "unsupported"), (N.LBM_ERR_STATE, "invalid state")):
        assert L.lbm_status_string(st).decode() == text


@pytest.mark.parametrize("field,value", [("quadrature", 7), ("quadrature", -1), ("nx", 0), ("ny", -3),
                                         ("storage", 6), ("collision", 4), ("force_kind", 4)])
def test_create_rejects_bad_descriptor_fields(lbm, L, field, value):
    assert _create(L, _desc(lbm, **{field: value})) == lbm._native.LBM_ERR_INVALID


def test_create_rejects_missing_arrays(lbm, L):
    N = lbm._native
    assert _create(L, _desc(lbm, force_kind=N.FORCE_FIELD)) == N.LBM_ERR_INVALID       # no force field
    assert _create(L, _desc(lbm, force_kind=N.FORCE_SHEAR)) == N.LBM_ERR_INVALID       # no coordinates
    assert _create(L, _desc(lbm, collision=N.ITERATIVE_INIT)) == N.LBM_ERR_INVALID     # no nonlinear term
    assert _create(L, _desc(lbm, nbc=1)) == N.LBM_ERR_INVALID                           # no BC array
    assert _create(L, _desc(lbm, nbc=N.MAX_BC + 1)) == N.LBM_ERR_INVALID
    h = C.c_void_p()
    assert L.lbm_create(C.byref(h), None) == N.LBM_ERR_INVALID
    assert L.lbm_create(None, C.byref(_desc(lbm))) == N.LBM_ERR_INVALID


def _with_bc(lbm, kind, direction, xs, ys, nx=8, ny=6):
    N = lbm._native
    arr = (N.LbmBC * 1)()
    arr[0].kind, arr[0].direction = kind, direction
    arr[0].x_lo, arr[0].x_hi = xs
    arr[0].y_lo, arr[0].y_hi = ys
    d = _desc(lbm, nx=nx, ny=ny, nbc=1)
    d.bcs = C.cast(arr, C.POINTER(N.LbmBC))
    return d, arr


def test_create_rejects_bad_boundary_conditions(lbm, L):
    N = lbm._native
    for kind, direction, xs, ys, status in (
            (5, N.NORTH, (1, 8), (1, 6), N.LBM_ERR_INVALID),             # unknown kind
            (N.BOUNCE_BACK, 4, (1, 8), (1, 6), N.LBM_ERR_INVALID),       # unknown direction
            (N.BOUNCE_BACK, N.NORTH, (0, 8), (1, 6), N.LBM_ERR_INVALID),  # x range below 1
            (N.BOUNCE_BACK, N.NORTH, (1, 9), (1, 6), N.LBM_ERR_INVALID),  # x range past nx
            (N.BOUNCE_BACK, N.SOUTH, (1, 8), (1, 7), N.LBM_ERR_INVALID),  # y range past ny
            (N.MOVING_WALL, N.SOUTH, (1, 8), (1, 6), N.LBM_ERR_UNSUPPORTED)):  # moving wall: North only
        d, keep = _with_bc(lbm, kind, direction, xs, ys)
        assert _create(L, d) == status, (kind, direction, xs, ys)


def test_create_rejects_weights_without_class_symmetry(lbm, L):
    d = _desc(lbm)
    d.weights[1] = d.weights[1] * (1 + 1e-9)  # one axis velocity off its class's weight
    assert _create(L, d) == lbm._native.LBM_ERR_INVALID


def test_null_handles(lbm, L):
    N = lbm._native
    out = np.zeros(16)
    assert L.lbm_step(None, 1, 0, 0.0) == N.LBM_ERR_INVALID
    assert L.lbm_upload(None, out.ctypes.data) == N.LBM_ERR_INVALID
    assert L.lbm_reduce(None, 0, None, out.ctypes.data_as(N._DP)) == N.LBM_ERR_INVALID
    assert L.lbm_set_stream(None, None) == N.LBM_ERR_INVALID
    assert L.lbm_initialize_fields(None, None, None, None, None, None, None, None, 0.0, 0) == N.LBM_ERR_INVALID
    assert L.lbm_last_error(None).decode() == "null context"
    L.lbm_destroy(None)
    h = C.c_void_p()
    assert L.lbm_batch_create(C.byref(h), None, 1) == N.LBM_ERR_INVALID
    arr = (C.c_void_p * 1)(None)
    assert L.lbm_batch_create(C.byref(h), arr, 0) == N.LBM_ERR_INVALID
    assert L.lbm_batch_create(C.byref(h), arr, 1) == N.LBM_ERR_INVALID
    assert L.lbm_batch_step(None, None) == N.LBM_ERR_INVALID
    assert L.lbm_batch_step_timed(None, None, None, None) == N.LBM_ERR_INVALID
    assert L.lbm_batch_reduce(None, 2, None, out.ctypes.data_as(N._DP)) == N.LBM_ERR_INVALID
    assert L.lbm_batch_last_error(None).decode() == "null batch"
    L.lbm_batch_destroy(None)


@pytest.mark.parametrize("nx,ny", [(2 ** 62 + 1, 4), (4, 2 ** 62 + 1), (2 ** 31, 1), (1, 2 ** 31),
                                   (2 ** 16, 2 ** 15)])
def test_lattice_sizes_that_wrap_or_exceed_32_bit_node_indices(lbm, L, nx, ny):
    """nx * ny formed in 64 bits wraps for (2^62 + 1) x 4 to 4 nodes; each factor is bounded
    before the product, so such pairs are refused like every lattice of 2^31 nodes or more."""
    N = lbm._native
    assert _create(L, _desc(lbm, nx=nx, ny=ny)) == N.LBM_ERR_INVALID
    q = lbm.D2Q9()
    w = np.asarray(q.weights, dtype=np.float64)
    fn = L.lbm_reduce_noalloc
    fn.argtypes = [C.c_int32, C.POINTER(C.c_double), C.c_double, C.c_int64, C.c_int64, C.c_void_p, C.c_int32,
                   C.POINTER(N.LbmAnalytic), C.c_void_p, C.c_void_p]
    fn.restype = C.c_int32
    dummy = np.zeros(16)  # never read: the sizes are refused before any pointer is used
    st = fn(q.qid, w.ctypes.data_as(C.POINTER(C.c_double)), q.speed_of_sound_squared, nx, ny,
            dummy.ctypes.data, N.REDUCE_CONSERVED, None, dummy.ctypes.data, None)
    assert st == N.LBM_ERR_INVALID
