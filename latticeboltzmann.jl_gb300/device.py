"""DeviceLattice: one liblbm_gb300 context (the populations of one lattice on the GPU plus
its quadrature, collision model and boundary list), wrapped for Python callers.

Populations cross the boundary in the reference's Julia layout f[x, y, i]; in numpy that is
a C-contiguous float64 array of shape (Q, NY, NX).
"""
from __future__ import annotations

import ctypes as C
import weakref

import numpy as np

from . import _native as N
from .boundary_conditions import BounceBack, MovingWall
from .collision_models import MRT, SRT, TRT, IterativeInitializationCollisionModel


def _as_f64(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if shape is not None and a.shape != shape:
        raise ValueError(f"expected shape {shape}, got {a.shape}")
    return a


class DeviceLattice:
    """A lattice of nx x ny nodes with populations resident in HBM.

    force: None | ("constant", (Fx, Fy)) | ("field", array (2, NY, NX)) |
           ("shear", [c0..c5], x_coords, y_coords)
    storage: "f64" | "df64dev" (float-float deviation) | "f32dev" | "f16dev" | "f32sr" (FP32 deviation,
             float-float arithmetic, stochastically rounded stores) | "f64dd" (FP64 storage, float-float
             arithmetic on the deviation)
    nonlinear: the (Q, NY, NX) term of the iterative-initialisation collision model
    """

    def __init__(self, q, nx, ny, collision_model, bcs=(), force=None, storage="f64", nonlinear=None):
        L = N.lib()
        self.q = q
        self.nx, self.ny = int(nx), int(ny)
        self.Q = q.Q
        self.shape = (self.Q, self.ny, self.nx)
        self.storage = storage
        d = N.LbmDesc()
        d.quadrature = q.qid
        for i, w in enumerate(q.weights):
            d.weights[i] = float(w)
        d.speed_of_sound_squared = q.speed_of_sound_squared
        cm = collision_model
        if isinstance(cm, SRT):
            d.collision, taus = N.SRT, [cm.τ]
        elif isinstance(cm, TRT):
            d.collision, taus = N.TRT, [cm.τ_symmetric, cm.τ_asymmetric]
        elif isinstance(cm, MRT):
            d.collision = N.MRT
            taus = list(cm.τs) + [1.0] * max(0, 4 - len(cm.τs))
        elif isinstance(cm, IterativeInitializationCollisionModel):
            d.collision, taus = N.ITERATIVE_INIT, [cm.τ]
        else:
            raise TypeError(f"unsupported collision model {cm!r}")
        for k, t in enumerate(taus[:4]):
            d.tau[k] = float(t)
        self._keep = []
        d.force_kind = N.FORCE_NONE
        if force is not None:
            kind = force[0]
            if kind == "constant":
                d.force_kind = N.FORCE_CONSTANT
                d.force[0], d.force[1] = float(force[1][0]), float(force[1][1])
            elif kind == "field":
                ff = _as_f64(force[1], (2, self.ny, self.nx))
                self._keep.append(ff)
                d.force_kind = N.FORCE_FIELD
                d.force_field = ff.ctypes.data_as(N._DP)
            elif kind == "shear":
                xr = _as_f64(force[2], (self.nx,))
                yr = _as_f64(force[3], (self.ny,))
                self._keep += [xr, yr]
                d.force_kind = N.FORCE_SHEAR
                for k in range(6):
                    d.shear[k] = float(force[1][k])
                d.x_coords = xr.ctypes.data_as(N._DP)
                d.y_coords = yr.ctypes.data_as(N._DP)
            else:
                raise ValueError(f"unknown force kind {kind}")
        if nonlinear is not None:
            nl = _as_f64(nonlinear, self.shape)
            self._keep.append(nl)
            d.nonlinear = nl.ctypes.data_as(N._DP)
        bcs = list(bcs)
        if len(bcs) > N.MAX_BC:
            raise ValueError(f"at most {N.MAX_BC} boundary conditions")
        arr = (N.LbmBC * max(1, len(bcs)))()
        for k, b in enumerate(bcs):
            e = arr[k]
            e.kind = N.BOUNCE_BACK if isinstance(b, BounceBack) else N.MOVING_WALL
            e.direction = b.direction.code
            e.x_lo, e.x_hi = b.xs
            e.y_lo, e.y_hi = b.ys
            if isinstance(b, MovingWall):
                e.u[0], e.u[1] = b.u
                e.rho, e.T = b.ρ, b.T
        self._keep.append(arr)
        d.nbc = len(bcs)
        d.bcs = C.cast(arr, C.POINTER(N.LbmBC))
        d.nx, d.ny = self.nx, self.ny
        d.storage = N.STORAGE_IDS[storage]
        h = C.c_void_p()
        st = L.lbm_create(C.byref(h), C.byref(d))
        if st != N.LBM_OK:
            raise N.LbmError(st, f"lbm_create: {L.lbm_status_string(st).decode()}")
        self.h = h
        self._keep = []  # the library copied what it needs
        self.prefetched = {}  # reduction kind -> sums supplied by a batched reduction

    # ---- lifetime ----------------------------------------------------------------------
    def close(self):
        # a batch holds this context without owning it (and may have lent it its stream), so any
        # open batch of this lattice goes first
        for b in list(getattr(self, "_batches", ())):
            b.close()
        if getattr(self, "h", None):
            N.lib().lbm_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_handle: int | None):
        N.check(self.h, N.lib().lbm_set_stream(self.h, stream_handle or None))

    def synchronize(self):
        N.check(self.h, N.lib().lbm_synchronize(self.h))

    # ---- populations -------------------------------------------------------------------
    def upload(self, f):
        if hasattr(f, "data_ptr"):  # torch tensor
            if f.is_cuda:
                N.check(self.h, N.lib().lbm_upload_device(self.h, f.data_ptr()))
                return
            N.check(self.h, N.lib().lbm_upload(self.h, f.data_ptr()))
            return
        f = _as_f64(f, self.shape)
        N.check(self.h, N.lib().lbm_upload(self.h, f.ctypes.data))

    def initialize_fields(self, rho=None, ux=None, uy=None, T=None, S=None, coef=0.0, times_rho=False):
        """lbm_initialize_fields: the initial state from macroscopic (NY, NX) planes, computed on
        the device (None: ρ = 1, u = 0, T = 1, no stress term; S = (sxx, sxy, syy))."""
        shp = (self.ny, self.nx)
        keep = []

        def ptr(a):
            if a is None:
                return None
            a = _as_f64(np.broadcast_to(a, shp))
            keep.append(a)
            return a.ctypes.data_as(N._DP)
        s = (None, None, None) if S is None else S
        N.check(self.h, N.lib().lbm_initialize_fields(self.h, ptr(rho), ptr(ux), ptr(uy), ptr(T), ptr(s[0]),
                                                       ptr(s[1]), ptr(s[2]), float(coef), 1 if times_rho else 0))

    def download(self, out=None):
        if out is not None and hasattr(out, "data_ptr"):
            fn = N.lib().lbm_download_device if out.is_cuda else N.lib().lbm_download
            N.check(self.h, fn(self.h, out.data_ptr()))
            return out
        out = np.empty(self.shape) if out is None else out
        N.check(self.h, N.lib().lbm_download(self.h, out.ctypes.data))
        return out

    def step(self, nsteps: int, t0: int = 0, dt: float = 0.0):
        N.check(self.h, N.lib().lbm_step(self.h, int(nsteps), int(t0), float(dt)))

    def last_launch_count(self) -> int:
        return int(N.lib().lbm_last_launch_count(self.h))

    # ---- reductions --------------------------------------------------------------------
    def reduce(self, kind, fields=None, tau=0.0, u_max=1.0, area=0.0):
        pre = self.prefetched.pop(kind, None)
        if pre is not None:  # computed for this lattice by a batched reduction (simulate_batch)
            return pre
        out = np.zeros(16)
        an = None
        keep = []
        if fields is not None:
            an = N.LbmAnalytic()
            for name in ("rho", "ux", "uy", "p", "sxx", "syx", "sxy", "syy"):
                a = fields.get(name)
                if a is not None:
                    if hasattr(a, "data_ptr"):
                        an.on_device = 1
                        setattr(an, name, C.cast(C.c_void_p(a.data_ptr()), N._DP))
                    else:
                        a = _as_f64(a, (self.ny, self.nx))
                        keep.append(a)
                        setattr(an, name, a.ctypes.data_as(N._DP))
            an.tau, an.u_max, an.area = float(tau), float(u_max), float(area)
        st = N.lib().lbm_reduce(self.h, int(kind), C.byref(an) if an is not None else None,
                                out.ctypes.data_as(N._DP))
        N.check(self.h, st)
        return out[: N.REDUCE_K[kind]]

    def density_at(self, x: int, y: int) -> float:
        out = np.zeros(16)
        out[0], out[1] = x, y
        N.check(self.h, N.lib().lbm_reduce(self.h, N.REDUCE_DENSITY_AT, None, out.ctypes.data_as(N._DP)))
        return float(out[0])

    def conserved(self):
        """Σρ, Σρux, Σρuy over the lattice; raises on non-finite populations."""
        return self.reduce(N.REDUCE_CONSERVED)[:3]

    def macroscopic(self):
        rho = np.empty((self.ny, self.nx))
        ux = np.empty((self.ny, self.nx))
        uy = np.empty((self.ny, self.nx))
        N.check(self.h, N.lib().lbm_macroscopic(self.h, rho.ctypes.data, ux.ctypes.data, uy.ctypes.data))
        return rho, ux, uy

    # ---- single operators on caller-owned device arrays --------------------------------
    def collide_device(self, f_in, f_out, time=0.0):
        N.check(self.h, N.lib().lbm_collide_device(self.h, N.ptr(f_in), N.ptr(f_out), float(time)))

    def stream_device(self, f, f_new):
        N.check(self.h, N.lib().lbm_stream_device(self.h, N.ptr(f), N.ptr(f_new)))

    def apply_bcs_device(self, f_new, f_old):
        N.check(self.h, N.lib().lbm_apply_bcs_device(self.h, N.ptr(f_new), N.ptr(f_old)))


class DeviceBatch:
    """Several DeviceLattices advanced together: member k takes nsteps[k] steps (lbm_batch_*).
    Small members take all their steps of a call in one block-resident launch (a thread-block
    cluster per member, its populations in shared memory); the others are issued as one CUDA graph
    with one kernel per global step over every member still running.  `schedule` picks the small
    members: "measured" (the table tune_batch.py measured on the GPU, batch_schedule.json), None
    (every member on the graph path) or an explicit {velocity set: {"resident_max_nodes",
    "nodes_per_block"}} mapping; the results are the same bits either way.  Members must share
    storage (f64, df64dev or f32dev) and collision kind (SRT, TRT or MRT); members with a
    time-dependent force are stepped with their times (step(nsteps, t0, dt)).  The batch holds its
    members' contexts without owning them: close the batch before any member."""

    def __init__(self, lattices, schedule="measured"):
        L = N.lib()
        self.lattices = list(lattices)
        if any(not getattr(lat, "h", None) for lat in self.lattices):
            raise ValueError("a batch member is closed")
        arr = (C.c_void_p * len(self.lattices))(*[lat.h.value for lat in self.lattices])
        h = C.c_void_p()
        st = L.lbm_batch_create(C.byref(h), arr, len(self.lattices))
        if st != N.LBM_OK:
            raise N.LbmError(st, "lbm_batch_create: members must share storage and collision kind (SRT, TRT, MRT), "
                                 "use f64 / df64dev / f32dev, and each appear once")
        self.h = h
        self.set_schedule(schedule)
        for lat in self.lattices:  # weak: the batch's references keep the members, not the other way
            if not hasattr(lat, "_batches"):
                lat._batches = weakref.WeakSet()
            lat._batches.add(self)

    def _open(self):
        """The batch and every member still open: the library holds the members' contexts, so a
        member closed first would leave it a freed context."""
        if not getattr(self, "h", None):
            raise ValueError("the batch is closed")
        for k, lat in enumerate(self.lattices):
            if not getattr(lat, "h", None):
                raise ValueError(f"batch member {k} was closed before its batch")

    def _check(self, st):
        if st != N.LBM_OK:
            raise N.LbmError(st, N.lib().lbm_batch_last_error(self.h).decode())

    def step(self, nsteps, t0=None, dt=None):
        """Advance member k by nsteps[k] steps.  With t0 and dt (one per member), step j of member k
        runs at time (t0[k] + j) dt[k], which members with a time-dependent force need."""
        self._open()
        ns = np.ascontiguousarray(nsteps, dtype=np.int64)
        if ns.shape != (len(self.lattices),):
            raise ValueError("one step count per member")
        if t0 is None and dt is None:
            self._check(N.lib().lbm_batch_step(self.h, ns.ctypes.data_as(C.POINTER(C.c_int64))))
            return
        t0a = np.ascontiguousarray(np.broadcast_to(np.asarray(t0, dtype=np.int64), ns.shape))
        dta = np.ascontiguousarray(np.broadcast_to(np.asarray(dt, dtype=np.float64), ns.shape))
        self._check(N.lib().lbm_batch_step_timed(self.h, ns.ctypes.data_as(C.POINTER(C.c_int64)),
                                                  t0a.ctypes.data_as(C.POINTER(C.c_int64)),
                                                  dta.ctypes.data_as(N._DP)))

    def set_stream(self, stream_handle):
        self._open()
        self._check(N.lib().lbm_batch_set_stream(self.h, stream_handle or None))

    def set_schedule(self, schedule="measured"):
        """lbm_batch_set_schedule: which members step block-resident (see the class docstring)."""
        from .batch_schedule import schedule_for
        self._open()
        st = schedule_for(self.lattices[0].storage, schedule)
        self._check(N.lib().lbm_batch_set_schedule(self.h, C.byref(st) if st is not None else None))

    def synchronize(self):
        self._open()
        self._check(N.lib().lbm_batch_synchronize(self.h))

    def last_launch_count(self) -> int:
        return int(N.lib().lbm_batch_last_launch_count(self.h))

    def reduce(self, kind, select=None):
        """lbm_batch_reduce: the (members, K) sums of a stop-criterion reduction of the selected
        members (all when select is None; rows of unselected members are zero)."""
        self._open()
        out = np.zeros((len(self.lattices), 16))
        sel = None
        if select is not None:
            sel = np.ascontiguousarray(select, dtype=np.uint8)
            if sel.shape != (len(self.lattices),):
                raise ValueError("one select flag per member")
        self._check(N.lib().lbm_batch_reduce(self.h, int(kind),
                                             sel.ctypes.data_as(C.POINTER(C.c_uint8)) if sel is not None else None,
                                             out.ctypes.data_as(N._DP)))
        return out[:, : N.REDUCE_K[kind]]

    def reduce_fields(self, kind, inputs):
        """lbm_batch_reduce_fields: the TRACK_ERRORS / COMPARE sums of the members for which
        `inputs[k]` = (fields dict of (NY, NX) host planes, tau, u_max, area) is given (None:
        not selected); rows of unselected members are zero."""
        self._open()
        n = len(self.lattices)
        sel = np.zeros(n, dtype=np.uint8)
        an = (N.LbmAnalytic * n)()
        keep = []
        for k, inp in enumerate(inputs):
            if inp is None:
                continue
            fields, tau, u_max, area = inp
            lat = self.lattices[k]
            for name in ("rho", "ux", "uy", "p", "sxx", "syx", "sxy", "syy"):
                a = fields.get(name)
                if a is not None:
                    a = _as_f64(a, (lat.ny, lat.nx))
                    keep.append(a)
                    setattr(an[k], name, a.ctypes.data_as(N._DP))
            an[k].tau, an[k].u_max, an[k].area = float(tau), float(u_max), float(area)
            sel[k] = 1
        out = np.zeros((n, 16))
        self._check(N.lib().lbm_batch_reduce_fields(self.h, int(kind), sel.ctypes.data_as(C.POINTER(C.c_uint8)), an,
                                                    out.ctypes.data_as(N._DP)))
        return out[:, : N.REDUCE_K[kind]]

    def share_stream(self):
        """lbm_batch_share_stream: members issue their own work on the batch's stream."""
        self._open()
        self._check(N.lib().lbm_batch_share_stream(self.h))

    def close(self):
        if getattr(self, "h", None):
            N.lib().lbm_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
