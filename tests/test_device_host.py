"""Host-side lifetime rules of DeviceBatch (no GPU): the library holds a batch's member contexts
without owning them, so a batch refuses calls once a member is closed, and closing a member first
closes every open batch that holds it."""
import ctypes as C
import weakref

import numpy as np
import pytest


class _Closed:
    h = None


def test_batch_refuses_calls_after_a_member_closed(lbm):
    DeviceBatch = lbm.device.DeviceBatch
    b = object.__new__(DeviceBatch)
    b.h = C.c_void_p(1)  # never passed to the library: every call checks the members first
    b.lattices = [_Closed(), _Closed()]
    try:
        for call in (lambda: b.step([1, 1]), lambda: b.step([1, 1], [0, 0], [0.1, 0.1]), b.synchronize,
                     lambda: b.reduce(0), lambda: b.reduce_fields(0, [None, None]), b.share_stream,
                     lambda: b.set_stream(None)):
            with pytest.raises(ValueError, match="closed before its batch"):
                call()
    finally:
        b.h = None
    with pytest.raises(ValueError, match="batch is closed"):
        b.step([1, 1])


def test_closing_a_member_closes_its_batches_first(lbm):
    DeviceLattice = lbm.device.DeviceLattice
    order = []

    class _Batch:
        def close(self):
            order.append("batch")

    batches = [_Batch(), _Batch()]
    lat = object.__new__(DeviceLattice)
    lat.h = None  # no context: only the batch ordering runs
    lat._batches = weakref.WeakSet(batches)
    lat.close()
    assert order == ["batch", "batch"]


def test_batch_of_a_closed_lattice_is_refused(lbm):
    with pytest.raises(ValueError, match="member is closed"):
        lbm.device.DeviceBatch([_Closed()])


def test_adjoint_run_checks_its_inputs_before_the_library(lbm):
    AdjointProblem = lbm.adjoint.AdjointProblem
    a = object.__new__(AdjointProblem)
    a.h, a.nx, a.ny = None, 8, 6
    a.lattice = _Closed()
    a.lattice.close = lambda: None
    with pytest.raises(ValueError, match="closed"):
        a.run(np.zeros((2, 6, 8)), np.zeros((2, 6, 8)))
    a.h = C.c_void_p(1)  # never passed to the library: the shapes are checked first
    try:
        with pytest.raises(ValueError, match="shape"):
            a.run(np.zeros((2, 8, 6)), np.zeros((2, 8, 6)))
        with pytest.raises(ValueError, match="shape"):
            a.run(np.zeros((2, 6, 8)), np.zeros((2, 6, 7)))
    finally:
        a.h = None
