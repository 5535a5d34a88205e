"""Error behaviour of the C ABI on a live context: every misuse returns its documented status,
records a message, and leaves the context usable."""
import ctypes as C

import numpy as np
import pytest

from gpu_cases import wave_field

pytestmark = pytest.mark.gpu


def _lattice(lbm, qname="D2Q9", storage="f64", cm=None, nx=12, ny=10):
    q = lbm.Quadratures[qname]
    return lbm.DeviceLattice(q, nx, ny, cm or lbm.TRT.fields(0.8, 1.1), (), storage=storage)


def test_state_and_argument_errors(lbm_gpu):
    lbm = lbm_gpu
    N = lbm._native
    L = N.lib()
    lat = _lattice(lbm)
    assert L.lbm_step(lat.h, 3, 0, 0.0) == N.LBM_ERR_STATE            # nothing uploaded yet
    assert b"no state" in L.lbm_last_error(lat.h)
    out = np.zeros(16)
    assert L.lbm_reduce(lat.h, N.REDUCE_CONSERVED, None, out.ctypes.data_as(N._DP)) == N.LBM_ERR_STATE
    lat.initialize_fields()
    assert L.lbm_step(lat.h, -1, 0, 0.0) == N.LBM_ERR_INVALID
    assert L.lbm_reduce(lat.h, 99, None, out.ctypes.data_as(N._DP)) == N.LBM_ERR_INVALID
    assert L.lbm_reduce(lat.h, N.REDUCE_TRACK_ERRORS, None, out.ctypes.data_as(N._DP)) == N.LBM_ERR_INVALID
    out[0], out[1] = 12, 0  # node x out of range
    assert L.lbm_reduce(lat.h, N.REDUCE_DENSITY_AT, None, out.ctypes.data_as(N._DP)) == N.LBM_ERR_INVALID
    sxx = np.zeros((10, 12))
    assert L.lbm_initialize_fields(lat.h, None, None, None, None, sxx.ctypes.data_as(N._DP), None, None, 1.0,
                                   0) == N.LBM_ERR_INVALID
    # the context is still usable
    lat.step(5)
    assert abs(lat.conserved()[0] - 12 * 10) < 1e-12
    lat.close()


def test_failed_allocation_is_not_reported_again(lbm_gpu):
    """A lattice too large for the device (D2Q37 FP64, 46000 x 46000 nodes: 626 GB per population
    array, under the 2^31-node limit) is refused with LBM_ERR_NOMEM at its first allocation; the
    failed allocation stays out of the launch checks of later, unrelated calls."""
    lbm = lbm_gpu
    N = lbm._native
    with pytest.raises(N.LbmError) as e:
        _lattice(lbm, "D2Q37", "f64", lbm.SRT(0.8), nx=46000, ny=46000)
    assert e.value.status == N.LBM_ERR_NOMEM
    lat = _lattice(lbm)
    lat.initialize_fields()
    lat.step(5)
    assert abs(lat.conserved()[0] - 12 * 10) < 1e-12
    lat.close()


def test_non_finite_populations_are_reported(lbm_gpu):
    lbm = lbm_gpu
    N = lbm._native
    lat = _lattice(lbm)
    f = np.ascontiguousarray(wave_field(lbm.D2Q9(), 12, 10, seed=3))
    f[4, 3, 5] = np.nan
    lat.upload(f)
    with pytest.raises(N.LbmError) as e:
        lat.conserved()
    assert e.value.status == N.LBM_ERR_NONFINITE
    lat.close()


def test_unsupported_combinations(lbm_gpu):
    lbm = lbm_gpu
    N = lbm._native
    L = N.lib()
    a = _lattice(lbm, storage="f64")
    b = _lattice(lbm, storage="f32dev")
    with pytest.raises(N.LbmError):            # members must share the storage
        lbm.DeviceBatch([a, b])
    c = _lattice(lbm, cm=lbm.SRT(0.8))
    with pytest.raises(N.LbmError):            # ... and the collision kind
        lbm.DeviceBatch([a, c])
    with pytest.raises(N.LbmError):            # ... and appear once
        lbm.DeviceBatch([a, a])
    h = C.c_void_p()
    d17 = _lattice(lbm, "D2Q17")
    assert L.lbm_adjoint_create(C.byref(h), d17.h, 10, 0) == N.LBM_ERR_UNSUPPORTED
    assert b"adjoint" in L.lbm_last_error(d17.h)
    f16 = _lattice(lbm, storage="f16dev")
    assert L.lbm_collide_device(f16.h, None, None, 0.0) in (N.LBM_ERR_INVALID, N.LBM_ERR_UNSUPPORTED)
    for lat in (a, b, c, d17, f16):
        lat.close()


@pytest.mark.parametrize("storage", ["f32sr", "f64dd", "f16dev"])
def test_single_lattice_storages_refuse_batches_and_the_adjoint(lbm_gpu, storage):
    """The stochastically rounded FP32, the FP64-storage float-float and the FP16 storages step
    single lattices only: a batch of them and an adjoint on them are refused with
    LBM_ERR_UNSUPPORTED, and the lattices stay usable."""
    lbm = lbm_gpu
    N = lbm._native
    L = N.lib()
    a, b = _lattice(lbm, storage=storage), _lattice(lbm, storage=storage)
    with pytest.raises(N.LbmError) as err:
        lbm.DeviceBatch([a, b])
    assert err.value.status == N.LBM_ERR_UNSUPPORTED
    h = C.c_void_p()
    assert L.lbm_adjoint_create(C.byref(h), a.h, 10, 0) == N.LBM_ERR_UNSUPPORTED
    assert b"adjoint" in L.lbm_last_error(a.h)
    a.initialize_fields()
    a.step(3)
    assert np.all(np.isfinite(a.download()))
    a.close()
    b.close()
