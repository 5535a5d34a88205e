"""The GPU model type and the time loop: a drop-in for the reference's
LatticeBoltzmannModel / simulate (src/lattice_boltzmann_model.jl:1-110).

`simulate(model, time)` keeps the reference's loop semantics -- for every t in `time`:
collide!(time = tΔt), stream!, apply!(bcs), then next!(model, t + 1), stopping when next!
returns true, and a final next!(model, last + 1) -- but issues the steps between two
processing events as one batch of fused device kernels (lbm_step), so the three lattice
passes of the reference become one kernel per step and no step waits for the host.
"""
from __future__ import annotations

import numpy as np

from . import _native as N
from .collision_models import IterativeInitializationCollisionModel, SRT, make_collision_model
from .device import DeviceLattice
from .initial_conditions import default_strategy, initial_fields, initialize
from .problems import DecayingShearFlow, PoiseuilleFlow, CouetteFlow, lattice_force_field, problem_range
from .processing_methods import NoProcessing, ProcessIterativeInitialization, ProcessingMethod


def _force_descriptor(cm, q, problem):
    """The device form of the collision model's force closure
    (x_idx, y_idx, t) -> lattice_force(problem, x_idx, y_idx, t)."""
    if cm.force is None:
        return None
    if cm.force != "problem":
        raise TypeError("a collision-model force is either None or the problem's lattice_force")
    if isinstance(problem, DecayingShearFlow) and problem.static:
        xr, yr, _, _ = problem_range(problem)
        return ("shear", problem.shear_force_params(), xr, yr)
    if getattr(problem, "force_is_time_dependent", False):
        raise NotImplementedError("time-dependent forces other than DecayingShearFlow's are not provided")
    if isinstance(problem, (PoiseuilleFlow, CouetteFlow)):  # uniform: the first node's force is every node's
        F = lattice_force_field(problem, 0.0, nodes=1)
        return ("constant", (float(F[0].flat[0]), float(F[1].flat[0])))
    F = lattice_force_field(problem, 0.0)
    if np.all(F[0] == F[0].flat[0]) and np.all(F[1] == F[1].flat[0]):
        return ("constant", (float(F[0].flat[0]), float(F[1].flat[0])))
    return ("field", F)


class LatticeBoltzmannModel:
    """LatticeBoltzmannModel(problem, q; collision_model=SRT, initialization_strategy, process_method)
    with the populations resident on the GPU.  `storage` selects FP64 ("f64"), the float-float
    deviation storage ("df64dev", FP64-class, FP32 pipes), the FP32 / FP16 deviation storage
    ("f32dev" / "f16dev"), the FP32 deviation storage with float-float arithmetic and
    stochastically rounded stores ("f32sr"), or FP64 storage with float-float arithmetic on the
    deviation ("f64dd").  Closed-form initial conditions are built on the
    device from their macroscopic planes unless `device_init` is False or `f0` (shape (Q, NY, NX))
    is given."""

    def __init__(self, problem, quadrature, collision_model=SRT, initialization_strategy=None,
                 process_method=None, storage="f64", f0=None, device_init=True):
        q = quadrature
        self.quadrature = q
        self.problem = problem
        strategy = default_strategy(problem) if initialization_strategy is None else initialization_strategy
        self.collision_model = make_collision_model(collision_model, q, problem)
        self.boundary_conditions = problem.boundary_conditions()
        self.processing_method = process_method if process_method is not None else NoProcessing(problem)
        # closed-form initial conditions are built on the device from their macroscopic planes
        # (lbm_initialize_fields); the rest, and explicit f0, are uploaded
        fields = initial_fields(strategy, q, problem) if f0 is None and device_init else None
        f = None
        if fields is None:
            f = initialize(strategy, q, problem, collision_model) if f0 is None else f0
        force = _force_descriptor(self.collision_model, q, problem)
        self.lattice = DeviceLattice(q, problem.NX, problem.NY, self.collision_model, self.boundary_conditions,
                                     force=force, storage=storage)
        if fields is None:
            self.lattice.upload(f)
        else:
            self.lattice.initialize_fields(**fields)

    @classmethod
    def from_parts(cls, quadrature, f0, collision_model, boundary_conditions=(), force=None, storage="f64",
                   process_method=None, problem=None):
        """A model from explicit parts (no problem object needed): the populations f0 of shape
        (Q, NY, NX), a collision model instance, a BC list and a device force descriptor."""
        m = cls.__new__(cls)
        m.quadrature = quadrature
        m.problem = problem
        m.collision_model = collision_model
        m.boundary_conditions = list(boundary_conditions)
        m.processing_method = process_method if process_method is not None else NoProcessing(problem)
        f0 = np.ascontiguousarray(f0, dtype=np.float64)
        _, ny, nx = f0.shape
        m.lattice = DeviceLattice(quadrature, nx, ny, collision_model, m.boundary_conditions, force=force,
                                  storage=storage)
        m.lattice.upload(f0)
        return m

    @property
    def f_stream(self):
        """The populations the reference's next! observes, downloaded as (Q, NY, NX) float64."""
        return self.lattice.download()

    def close(self):
        self.lattice.close()


def _time_bounds(time):
    if isinstance(time, range):
        if time.step != 1:
            raise ValueError("time ranges must have step 1")
        return time.start, time.stop - 1
    first, last = time
    return int(first), int(last)


def run_steps(model, first: int, last: int):
    """collide! -> stream! -> apply! for t = first..last with no processing (one device batch)."""
    pm = model.processing_method
    dt = pm.problem.delta_t() if getattr(pm, "problem", None) is not None else 0.0
    if last >= first:
        model.lattice.step(last - first + 1, first, dt)


def simulate_model(model, time):
    """simulate(model, time) (lattice_boltzmann_model.jl:60-77).  `time` is a Python range
    or an inclusive (first, last) pair, like Julia's first:last."""
    first, last = _time_bounds(time)
    pm = model.processing_method
    dt = pm.problem.delta_t() if getattr(pm, "problem", None) is not None else 0.0
    t = first
    while t <= last:
        ev = pm.next_event(t + 1)
        if ev is None or ev > last + 1:
            n = last - t + 1
        else:
            n = max(1, ev - t)
        model.lattice.step(n, t, dt)
        t += n
        if ev is not None and ev == t and pm.next(model, t):
            return model
    pm.next(model, last + 1)
    return model


def simulate_batch(models, times):
    """simulate(model, time) (lattice_boltzmann_model.jl:60-77) for many models at once, e.g. the
    points of a parameter sweep or a convergence study.  Each model follows exactly the loop of
    simulate_model -- its own steps, its own next! events, its own stop -- but the members step
    together through one DeviceBatch (one CUDA graph per round, one kernel per global step), and
    the stop criteria's reductions of all members due at a round come from one batched
    reduction.  `times` is one range / (first, last) pair for all models or one per model."""
    from .device import DeviceBatch
    models = list(models)
    n = len(models)
    if isinstance(times, (range, tuple)):
        times = [times] * n
    bounds = [_time_bounds(tm) for tm in times]
    t = [b[0] for b in bounds]
    last = [b[1] for b in bounds]
    pms = [m.processing_method for m in models]
    dts = np.array([pm.problem.delta_t() if getattr(pm, "problem", None) is not None else 0.0 for pm in pms])
    batch = DeviceBatch([m.lattice for m in models])
    batch.share_stream()
    if all(_vectorisable(pm) for pm in pms):
        try:
            _simulate_batch_vectorised(models, pms, bounds, batch, dts)
        finally:
            batch.close()
        return models
    stage = ["loop"] * n  # loop -> final (the last next!) -> done
    try:
        while True:
            nsteps = np.zeros(n, dtype=np.int64)
            events = [None] * n
            for k in range(n):
                if stage[k] != "loop":
                    continue
                if t[k] > last[k]:
                    stage[k] = "final"
                    continue
                ev = pms[k].next_event(t[k] + 1)
                nsteps[k] = last[k] - t[k] + 1 if ev is None or ev > last[k] + 1 else max(1, ev - t[k])
                events[k] = ev
            if nsteps.any():  # step j of member k at time (t[k] + j) Δt_k, as simulate_model steps it
                batch.step(nsteps, np.array(t, dtype=np.int64), dts)
            # members at an event (or at their final next!) and the stop reductions they will ask for
            acting = []
            for k in range(n):
                if nsteps[k]:
                    t[k] += int(nsteps[k])
                    if events[k] is not None and events[k] == t[k]:
                        acting.append((k, t[k]))
                elif stage[k] == "final":
                    acting.append((k, last[k] + 1))
            if not acting:
                if all(st == "done" for st in stage):
                    break
                continue
            due = {}
            for k, tk in acting:
                kind = pms[k].stop_reduction_due(tk)
                if kind is not None:
                    due.setdefault(kind, []).append(k)
            for kind, ks in due.items():
                sel = np.zeros(n, dtype=np.uint8)
                sel[ks] = 1
                rows = batch.reduce(kind, sel)
                for k in ks:
                    models[k].lattice.prefetched[kind] = rows[k]
            for k, tk in acting:
                stop = pms[k].next(models[k], tk)
                models[k].lattice.prefetched.clear()
                if stage[k] == "final" or stop:
                    stage[k] = "done"
            if all(st == "done" for st in stage):
                break
    finally:
        batch.close()
    return models


def _vectorisable(pm):
    from .processing_methods import (CompareWithAnalyticalSolution, MeanVelocityStoppingCriteria,
                                     NoStoppingCriteria, TrackHydrodynamicErrors, VelocityConvergenceStoppingCriteria)
    return (type(pm) in (TrackHydrodynamicErrors, CompareWithAnalyticalSolution) and not pm.should_process and
            type(pm.stop_criteria) in (NoStoppingCriteria, MeanVelocityStoppingCriteria,
                                       VelocityConvergenceStoppingCriteria))


def _simulate_batch_vectorised(models, pms, bounds, batch, dts):
    """simulate_batch for TrackHydrodynamicErrors / CompareWithAnalyticalSolution without
    per-step processing, with the members' bookkeeping in arrays: their events (every 100 steps
    for a stop criterion, and n_steps) and their stop decisions are computed for all members at
    once, and a member's own next!(model, t) is called only where it does more than decide not
    to stop (a row is due, or it stops); a MeanVelocity criterion that does not stop keeps its
    new mean as next! would (stopping_criteria.jl:20-72).  The rows recorded in one round (the
    error norms of every member that stops or reaches n_steps) come from one batched reduction."""
    from .processing_methods import (CompareWithAnalyticalSolution, TrackHydrodynamicErrors, compare_inputs,
                                     track_inputs)
    n = len(models)
    t = np.array([b[0] for b in bounds], dtype=np.int64)
    last = np.array([b[1] for b in bounds], dtype=np.int64)
    nst = np.array([pm.n_steps for pm in pms], dtype=np.int64)
    kind = np.array([-1 if pm.stop_criteria.reduce_kind is None else pm.stop_criteria.reduce_kind for pm in pms])
    stop_on = kind >= 0
    tol = np.array([getattr(pm.stop_criteria, "tolerance", 0.0) for pm in pms])
    mean_old = np.array([getattr(pm.stop_criteria, "old_mean_velocity", 0.0) for pm in pms])
    stage = np.zeros(n, dtype=np.int8)  # 0: time loop, 1: the final next!(model, last + 1), 2: done
    big = np.iinfo(np.int64).max // 4
    while True:
        loop = stage == 0
        ended = loop & (t > last)
        stage[ended] = 1
        loop &= ~ended
        tf = t + 1
        ev = np.where(stop_on, ((tf + 99) // 100) * 100, big)
        ev = np.where(nst >= tf, np.minimum(ev, nst), ev)
        steps = np.where(ev > last + 1, last - t + 1, np.maximum(1, ev - t))
        steps = np.where(loop, steps, 0).astype(np.int64)
        if steps.any():
            batch.step(steps, t, dts)
        t = t + steps
        act_loop = loop & (ev == t)
        act_final = stage == 1
        tact = np.where(act_final, last + 1, t)
        acting = act_loop | act_final
        due = acting & stop_on & (tact % 100 == 0)
        stop = np.zeros(n, dtype=bool)
        rows = {}
        um = None
        for kd in np.unique(kind[due]):
            sel = due & (kind == kd)
            r = batch.reduce(int(kd), sel.astype(np.uint8))
            rows[int(kd)] = r
            with np.errstate(divide="ignore", invalid="ignore"):
                if kd == N.REDUCE_VELOCITY_CONVERGENCE:
                    conv = np.sqrt(r[:, 0]) / r[:, 1]
                    st = (conv < tol) | np.isnan(conv)
                else:
                    um = r[:, 0] / r[:, 1]
                    conv = np.abs(um / mean_old - 1)
                    st = (conv < tol) | np.isnan(um)
            stop[sel] = st[sel]
        call = acting & (stop | (tact == nst))
        # the rows these calls record: all members' error norms in one batched reduction per kind
        idx = np.flatnonzero(call)
        if idx.size:
            for rkind, cls, make in ((N.REDUCE_TRACK_ERRORS, TrackHydrodynamicErrors, track_inputs),
                                     (N.REDUCE_COMPARE, CompareWithAnalyticalSolution, compare_inputs)):
                inputs = [None] * n
                for k in idx:
                    if type(pms[k]) is cls:
                        pb = pms[k].problem
                        tk = int(tact[k])
                        inputs[k] = make(models[k], pb, tk if cls is TrackHydrodynamicErrors else tk * pb.delta_t())
                if any(x is not None for x in inputs):
                    rws = batch.reduce_fields(rkind, inputs)
                    for k in idx:
                        if inputs[k] is not None:
                            models[k].lattice.prefetched[rkind] = rws[k]
        for k in np.flatnonzero(call):
            lat = models[k].lattice
            if due[k]:
                lat.prefetched[int(kind[k])] = rows[int(kind[k])][k]
            stop[k] = bool(pms[k].next(models[k], int(tact[k])))
            lat.prefetched.clear()
            if kind[k] == N.REDUCE_MEAN_VELOCITY:
                mean_old[k] = pms[k].stop_criteria.old_mean_velocity
        kept = due & ~call & (kind == N.REDUCE_MEAN_VELOCITY)
        for k in np.flatnonzero(kept):
            mean_old[k] = um[k]
            pms[k].stop_criteria.old_mean_velocity = float(um[k])
        stage[act_final] = 2
        stage[act_loop & stop] = 2
        if (stage == 2).all():
            return


def simulate(problem_or_model, q=None, *, time=None, process_method=None, should_process=True,
             initialization_strategy=None, t_end=1.0, collision_model=SRT, storage="f64"):
    """Both entry points of the reference:
       simulate(model, time)                                   lattice_boltzmann_model.jl:60-77
       simulate(problem, q; process_method, should_process, initialization_strategy,
                t_end, collision_model)                        lattice_boltzmann_model.jl:34-59"""
    if isinstance(problem_or_model, LatticeBoltzmannModel):
        return simulate_model(problem_or_model, time)
    problem = problem_or_model
    dt = problem.delta_t()
    n_steps = int(round(t_end / dt))
    if process_method is None:
        process_method = ProcessingMethod(problem, should_process, n_steps)
    model = LatticeBoltzmannModel(problem, q, collision_model=collision_model,
                                  initialization_strategy=initialization_strategy,
                                  process_method=process_method, storage=storage)
    return simulate_model(model, range(0, n_steps + 1))


# ---------------------------------------------------------------------------------------
# Mei et al. iterative initialisation (initial_conditions/mei_et_al.jl:11-40) on the device
# ---------------------------------------------------------------------------------------
def iterative_nonlinear_term(q, problem):
    """nonlinear_term[x, y, i] = w_i ρ0 (a_H1 + a_H2 / 2) of the fixed velocity field
    (iterative_initialization.jl:12-40), shape (Q, NY, NX)."""
    from .problems import lattice_velocity, node_grid
    X, Y = node_grid(problem)
    ux, uy = lattice_velocity(q, problem, X, Y)
    usq = ux ** 2 + uy ** 2
    cs = q.speed_of_sound_squared
    out = np.empty((q.Q,) + X.shape)
    for i in range(q.Q):
        cu = 0.0 + q.abscissae[0, i] * ux + q.abscissae[1, i] * uy
        a1 = cs * cu
        a2 = cs ** 2 * (cu * cu) - cs * usq
        out[i] = q.weights[i] * 1.0 * (a1 + a2 / 2)
    return out


def mei_initialize(strategy, q, problem, max_steps=10000):
    f = np.ascontiguousarray(np.broadcast_to(q.weights[:, None, None], (q.Q, problem.NY, problem.NX)),
                             dtype=np.float64)
    cm = IterativeInitializationCollisionModel(strategy.τ)
    pm = ProcessIterativeInitialization(strategy.ϵ, problem)
    m = LatticeBoltzmannModel.__new__(LatticeBoltzmannModel)
    m.quadrature, m.problem, m.collision_model = q, problem, cm
    m.boundary_conditions = problem.boundary_conditions()
    m.processing_method = pm
    m.lattice = DeviceLattice(q, problem.NX, problem.NY, cm, m.boundary_conditions,
                              nonlinear=iterative_nonlinear_term(q, problem))
    m.lattice.upload(f)
    simulate_model(m, range(1, max_steps + 1))
    out = m.f_stream
    m.close()
    return out


# ---------------------------------------------------------------------------------------
# the reference's operator plugin points on caller-owned CUDA arrays
# ---------------------------------------------------------------------------------------
_op_cache = {}


def _op_lattice(cm, q, shape, bcs=(), problem=None):
    Q, ny, nx = shape
    key = (id(cm), q.name, ny, nx, tuple(map(repr, bcs)), id(problem))
    lat = _op_cache.get(key)
    if lat is None:
        force = _force_descriptor(cm, q, problem) if cm is not None and problem is not None else None
        lat = DeviceLattice(q, nx, ny, cm if cm is not None else SRT(1.0), bcs, force=force)
        _op_cache[key] = lat
    return lat


def collide(cm, q, f_in, f_out, time=0.0, problem=None):
    """collide!(cm, q, f_in, f_out; time) (collision_models.jl:19, srt.jl:18, trt.jl:42, mrt.jl:49)
    on CUDA float64 tensors of shape (Q, NY, NX)."""
    lat = _op_lattice(cm, q, tuple(f_in.shape), problem=problem)
    lat.collide_device(f_in, f_out, time)
    lat.synchronize()


def stream(q, f, f_new):
    """stream!(q, f, f_new): periodic pull (stream.jl:18-30) on CUDA float64 tensors."""
    lat = _op_lattice(None, q, tuple(f.shape))
    lat.stream_device(f, f_new)
    lat.synchronize()


def apply(bcs, q, f_new, f_old):
    """apply!(bcs, q, f_new, f_old) (boundary_conditions.jl:6-20) on CUDA float64 tensors."""
    lat = _op_lattice(None, q, tuple(f_new.shape), bcs=list(bcs))
    lat.apply_bcs_device(f_new, f_old)
    lat.synchronize()
