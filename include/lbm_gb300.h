/*
 * lbm_gb300.h -- C ABI of the GB300-native lattice-Boltzmann collide-stream library
 * (liblbm_gb300.so, hand-written CUDA for sm_103a).
 *
 * The library replaces the per-step hot path of LatticeBoltzmann.jl:
 *
 *   simulate(model, time)            src/lattice_boltzmann_model.jl:60-77
 *     collide!(model; time)          src/lattice_boltzmann_model.jl:84-92 -> collide!(cm, q, f_in, f_out)
 *     stream!(model)                 src/lattice_boltzmann_model.jl:94-96 -> stream!(q, f, f_new)
 *     apply_boundary_conditions!     src/lattice_boltzmann_model.jl:98-106 -> apply!(bcs, q, f_new, f_old)
 *     next!(model, t)                src/lattice_boltzmann_model.jl:108-110 (the reductions below)
 *
 * with one fused pull kernel per time step.  A host binding (Julia `ccall`, Python ctypes)
 * keeps the reference's problem / initial-condition / processing layer and passes plain data
 * across this boundary: tables, relaxation times, forces, boundary descriptors and the
 * distribution array in the reference's own layout f[x, y, i] (column-major Julia array,
 * i.e. element f[x + nx * (y + ny * i)] with 0-based indices), so `pointer(f::Array{Float64,3})`
 * passes straight through.
 *
 * Conventions
 *   - Every entry point returns LBM_OK (0) or a negative lbm_status; no exception crosses the
 *     ABI.  lbm_last_error(ctx) describes the last failure on that context.
 *   - A context owns all device memory it allocates; host pointers are only read or written
 *     during the call that receives them.
 *   - One context is used by one host thread at a time.  Work is issued on the context's
 *     stream (its own non-blocking stream, or the one given to lbm_set_stream); calls that
 *     return host data synchronise that stream, lbm_step does not.
 *   - Devices: a context lives on the device that was current when lbm_create ran.  Every call on
 *     a context (or a batch / adjoint built on it) makes that device current for its duration
 *     and makes the caller's current device current again before it returns.
 *     lbm_reduce_noalloc, which has no context, runs on the caller's current device.
 *   - A failure of a CUDA call inside the library (status LBM_ERR_CUDA or LBM_ERR_NOMEM) is read
 *     and cleared from the thread's last-error slot when it is returned; other failures leave
 *     that slot as the caller left it.
 */
#ifndef LBM_GB300_H
#define LBM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LBM_ABI_VERSION 1
#define LBM_MAX_Q 37
#define LBM_MAX_BC 8

typedef enum {
  LBM_OK = 0,
  LBM_ERR_INVALID = -1,     /* bad argument or descriptor */
  LBM_ERR_CUDA = -2,        /* a CUDA runtime call failed */
  LBM_ERR_NOMEM = -3,       /* device or pinned host allocation failed */
  LBM_ERR_UNSUPPORTED = -4, /* combination not provided (e.g. MRT with FP16 storage) */
  LBM_ERR_STATE = -5,       /* call out of order (e.g. step before upload) */
  LBM_ERR_NONFINITE = -6    /* a reduction met NaN / Inf */
} lbm_status;

/* Velocity sets, in the order of the reference's `Quadratures` tuple (src/quadratures.jl:30-38).
 * LBM_D2Q21 has 25 velocities, as the reference's D2Q21 (src/quadratures/D2Q21.jl:36-66). */
typedef enum { LBM_D2Q4 = 0, LBM_D2Q5, LBM_D2Q9, LBM_D2Q13, LBM_D2Q17, LBM_D2Q21, LBM_D2Q37 } lbm_quadrature;

/* Collision operators: SRT  src/collision_models/srt.jl:1-62
 *                      TRT  src/collision_models/trt.jl:1-97
 *                      MRT  src/collision_models/mrt.jl:1-118 (regularised / projected)
 *                      ITERATIVE_INIT  src/collision_models/iterative_initialization.jl:1-60 */
typedef enum { LBM_SRT = 0, LBM_TRT = 1, LBM_MRT = 2, LBM_ITERATIVE_INIT = 3 } lbm_collision_kind;

/* Device storage of the distributions.
 *   F64       f itself, FP64 arithmetic (GB300 runs FP64 at 1/64 of the FP32 rate)
 *   F32_DEV   the deviation g_i = f_i - w_i in FP32, FP32 arithmetic
 *   F16_DEV   g_i in FP16, FP32 arithmetic
 *   DF64_DEV  g_i as a float-float pair (8 bytes, a 48-bit significand on a value far
 *             smaller than f), float-float arithmetic on the FP32 pipes: FP64-class results
 *             at the FP64 storage traffic.
 *   F32_DEV_SR  g_i in FP32 (the F32_DEV traffic), float-float arithmetic, and each collision
 *             output stored with stochastic rounding (unbiased; a counter-based hash of node,
 *             population and time index draws the rounding, so runs are reproducible): the
 *             rounding of a small, steady increment (a body force) no longer accumulates.
 *             Single lattices only (batches and the adjoint refuse it).
 *   F64_DD    f in FP64 (the F64 bytes and values), float-float arithmetic on g = f - w: the FP64
 *             pipe only forms g on load and w + g on store.  Single lattices only. */
typedef enum {
  LBM_STORE_F64 = 0,
  LBM_STORE_F32_DEV = 1,
  LBM_STORE_F16_DEV = 2,
  LBM_STORE_DF64_DEV = 3,
  LBM_STORE_F32_DEV_SR = 4,
  LBM_STORE_F64_DD = 5
} lbm_storage;

/* Forcing, applied as the reference does: a velocity shift of the equilibrium, u + τ F
 * (srt.jl:52-54, trt.jl:76-79, mrt.jl:91-95).
 *   CONSTANT: (force[0], force[1]) at every node (PoiseuilleFlow, poiseuille.jl:72-82)
 *   FIELD:    a time-independent lattice force per node, force_field[x + nx*(y + ny*d)]
 *   SHEAR:    the time-dependent DecayingShearFlow force (decaying_shear_flow.jl:132-147):
 *             Fx = shear[0] * cos(shear[1] * y - shear[2] * t)
 *             Fy = shear[3] * cos(shear[4] * x - shear[5] * t)
 *             with x, y the node coordinates x_coords[x], y_coords[y] and t the step time. */
typedef enum { LBM_FORCE_NONE = 0, LBM_FORCE_CONSTANT = 1, LBM_FORCE_FIELD = 2, LBM_FORCE_SHEAR = 3 } lbm_force_kind;

/* Boundary conditions (src/boundary_conditions.jl:6-35), applied in list order after the
 * periodic stream, each reading the post-collision populations of the same node:
 *   BOUNCE_BACK  src/boundary_conditions/bounce_back.jl:1-72 (all four directions)
 *   MOVING_WALL  src/boundary_conditions/moving_wall.jl:1-38 (North only; like the
 *                reference it ignores x_lo..y_hi and covers the whole top wall) */
typedef enum { LBM_BOUNCE_BACK = 0, LBM_MOVING_WALL = 1 } lbm_bc_kind;
typedef enum { LBM_NORTH = 0, LBM_EAST = 1, LBM_SOUTH = 2, LBM_WEST = 3 } lbm_direction;

typedef struct {
  int32_t kind;       /* lbm_bc_kind */
  int32_t direction;  /* lbm_direction */
  int32_t x_lo, x_hi; /* the BC's xs, 1-based inclusive (Julia UnitRange) */
  int32_t y_lo, y_hi; /* the BC's ys, 1-based inclusive */
  double u[2];        /* MOVING_WALL: wall velocity */
  double rho;         /* MOVING_WALL: wall density */
  double T;           /* MOVING_WALL: wall temperature (unused by the reference's rule) */
} lbm_bc;

typedef struct {
  int32_t quadrature;             /* lbm_quadrature */
  double weights[LBM_MAX_Q];      /* w_i as the host quadrature holds them (q.weights) */
  double speed_of_sound_squared;  /* the reference field of that name, i.e. 1 / c_s^2 */
  int32_t collision;              /* lbm_collision_kind */
  double tau[4];                  /* SRT: τ | TRT: τ_symmetric, τ_asymmetric | MRT: τs[1..4] | iterative: τ */
  int32_t force_kind;             /* lbm_force_kind */
  double force[2];                /* CONSTANT */
  const double* force_field;      /* FIELD: host array nx*ny*2, copied at create */
  double shear[6];                /* SHEAR */
  const double* x_coords;         /* SHEAR: host array of nx node coordinates */
  const double* y_coords;         /* SHEAR: host array of ny node coordinates */
  const double* nonlinear;        /* ITERATIVE_INIT: host array nx*ny*Q of the precomputed
                                     nonlinear equilibrium term, copied at create */
  int32_t nbc;                    /* number of boundary conditions, <= LBM_MAX_BC */
  const lbm_bc* bcs;
  int64_t nx, ny;                 /* lattice size (Julia size(f, 1), size(f, 2)) */
  int32_t storage;                /* lbm_storage */
} lbm_desc;

typedef struct lbm_ctx lbm_ctx;

/* Library identity. */
int32_t lbm_abi_version(void);
const char* lbm_status_string(int32_t status);

/* Context lifetime.  Replaces LatticeBoltzmannModel(problem, q; ...) for the data it holds
 * (src/lattice_boltzmann_model.jl:1-33): the two population arrays, the quadrature, the
 * collision model and the boundary-condition list. */
int32_t lbm_create(lbm_ctx** ctx, const lbm_desc* desc);
void lbm_destroy(lbm_ctx* ctx);
const char* lbm_last_error(const lbm_ctx* ctx);
/* Issue the context's work on `stream` (a cudaStream_t); NULL restores the own stream. */
int32_t lbm_set_stream(lbm_ctx* ctx, void* stream);
int32_t lbm_synchronize(lbm_ctx* ctx);

/* Populations in and out, in the Julia layout f[x + nx*(y + ny*i)] (FP64).  The state is
 * the reference's `f_stream` (the array next!(pm, q, f, t) observes). */
int32_t lbm_upload(lbm_ctx* ctx, const double* f_host);
int32_t lbm_download(lbm_ctx* ctx, double* f_host);
int32_t lbm_upload_device(lbm_ctx* ctx, const double* f_device);
int32_t lbm_download_device(lbm_ctx* ctx, double* f_device);

/* The initial state computed on the device from macroscopic planes (host arrays of nx*ny
 * doubles, Julia layout), instead of uploading Q planes built on the host by
 * `initialize(strategy, q, problem)` (initial_conditions.jl:7-22):
 *   f_i = equilibrium(q, ρ, u, T)_i   the Hermite expansion of hermite.jl:10-33
 *       + stress_coef [· ρ when stress_times_rho] · w_i · H_2(c_i) : S,  S = [sxx sxy; sxy syy]
 * which covers AnalyticalEquilibrium (analytical_equilibrium.jl), AnalyticalEquilibriumAndOff-
 * Equilibrium (analytical_offequilibrium.jl:10-87, both forms), ConstantDensity and
 * AnalyticalVelocityAndStress, and ZeroVelocityInitialCondition (everything NULL: f = w).
 * rho / T NULL mean 1, ux / uy NULL mean 0; sxx, sxy, syy are all given or all NULL.
 * The state becomes f_stream, as after lbm_upload. */
int32_t lbm_initialize_fields(lbm_ctx* ctx, const double* rho, const double* ux, const double* uy, const double* T,
                              const double* sxx, const double* sxy, const double* syy, double stress_coef,
                              int32_t stress_times_rho);

/* `nsteps` iterations of the reference loop body for t = t0, ..., t0 + nsteps - 1:
 * collide!(time = t*dt) -> stream! -> apply!(bcs), as simulate(model, time) does
 * (src/lattice_boltzmann_model.jl:64-67).  Asynchronous on the context's stream. */
int32_t lbm_step(lbm_ctx* ctx, int64_t nsteps, int64_t t0, double dt);

/* Launch count of the last lbm_step call (kernels issued, for accounting). */
int64_t lbm_last_launch_count(const lbm_ctx* ctx);

/* ---- reductions for the processing methods (next!) --------------------------------------- */

/* Analytic fields for the error norms, host or device arrays of nx*ny each (Julia layout),
 * in the dimensionless units the reference compares in. */
typedef struct {
  const double* rho;  /* expected density */
  const double* ux;   /* expected velocity */
  const double* uy;
  const double* p;    /* expected pressure */
  const double* sxx;  /* expected deviatoric stress σ[1,1], σ[2,1], σ[1,2], σ[2,2] */
  const double* syx;
  const double* sxy;
  const double* syy;
  int32_t on_device;  /* 1: the pointers are device pointers */
  double tau;         /* τ = (1/c_s²)·ν used by the stress estimate (track_hydrodynamic_errors.jl:148,176) */
  double u_max;       /* dimensionless_velocity scale (problems.jl:110) */
  double area;        /* the `opp` cell area of CompareWithAnalyticalSolution (processing_methods.jl:234) */
} lbm_analytic;

/* Kinds of lbm_reduce:
 *   TRACK_ERRORS  sums of TrackHydrodynamicErrors.next! (track_hydrodynamic_errors.jl:104-203):
 *                 out[0..15] = Σ(ρ-ρ*)², Σ|u-u*|², Σ(p-p*)², Σ(σxx-σxx*)², Σ(σxy-σxy*)²,
 *                 Σ(σyy-σyy*)², Σ(σyx-σyx*)², Σ|u*|², Σσxx*², Σσyy*², Σσxy*², Σσyx*², Σp*²,
 *                 Σρ, Σρ(ux+uy), Σρ|u|²   (u dimensionless, σ scaled by 1/u_max²)
 *   COMPARE       sums of CompareWithAnalyticalSolution process! (processing_methods.jl:142-239):
 *                 out[0..11] = Σρ, Σρ(ux+uy), Σ(ke+T), Σke, ΣT, Σρ*, Σρ*(ux*+uy*), Σ(ke*+T*),
 *                 Σke*, ΣT*, area·Σ|u-u*|², area·Σ(p-p*)²
 *   MEAN_VELOCITY Σ ux and the node count (stopping_criteria.jl:34-56): out[0], out[1]
 *   VELOCITY_CONVERGENCE  Σ|u-u_old|², Σ|u_old|², then u_old := u (stopping_criteria.jl:88-115)
 *   DENSITY_AT    density of node (ix, iy) = (out[0], out[1]) on entry (density_convergence.jl:6-17)
 *   CONSERVED     Σρ, Σρux, Σρuy, number of non-finite populations (out[0..3])
 * Sums are FP64, taken in a fixed order (deterministic across runs). */
typedef enum {
  LBM_REDUCE_TRACK_ERRORS = 0,
  LBM_REDUCE_COMPARE = 1,
  LBM_REDUCE_MEAN_VELOCITY = 2,
  LBM_REDUCE_VELOCITY_CONVERGENCE = 3,
  LBM_REDUCE_DENSITY_AT = 4,
  LBM_REDUCE_CONSERVED = 5
} lbm_reduce_kind;

int32_t lbm_reduce(lbm_ctx* ctx, int32_t kind, const lbm_analytic* analytic, double* out);

/* Macroscopic fields of the current state, Julia layout, host arrays of nx*ny
 * (density / velocity!, src/velocity_distribution_function/moments.jl:1-19).  Any pointer
 * may be NULL. */
int32_t lbm_macroscopic(lbm_ctx* ctx, double* rho, double* ux, double* uy);

/* ---- single operators on caller-owned device arrays (FP64, Julia layout) ----------------
 * The reference's plugin points, for callers that keep their own arrays on the GPU.  They
 * use the context's quadrature, collision model and BC list; f_in / f_out etc. are device
 * pointers of nx*ny*Q doubles. */
int32_t lbm_collide_device(lbm_ctx* ctx, const double* f_in, double* f_out, double time); /* collide!(cm, q, f_in, f_out; time) */
int32_t lbm_stream_device(lbm_ctx* ctx, const double* f, double* f_new);                   /* stream!(q, f, f_new), periodic */
int32_t lbm_apply_bcs_device(lbm_ctx* ctx, double* f_new, const double* f_old);            /* apply!(bcs, q, f_new, f_old) */

/* ---- batches: many lattices in one CUDA graph ---------------------------------------------
 * A convergence study or a parameter sweep is a set of independent lattices (one `simulate` per
 * point in the reference, e.g. examples/notebooks/taylor_green_vortex.ipynb cell 3 and
 * examples/notebooks/trt_magic_parameter.ipynb).  A batch groups existing contexts (same
 * storage and collision model kind -- SRT, TRT or MRT --, any velocity set, FP64, float-float or
 * FP32-deviation storage) and advances member k
 * by nsteps[k] steps with ONE graph launch: one kernel per global step, covering every member
 * still running.  Members keep their buffers; upload / download / reduce them as usual before
 * and after (their streams are ordered against the batch).  The batch holds its members'
 * contexts without owning them: destroy the batch before any of its members. */
typedef struct lbm_batch lbm_batch;
int32_t lbm_batch_create(lbm_batch** batch, lbm_ctx* const* members, int32_t count);  /* each context at most once */
void lbm_batch_destroy(lbm_batch* batch);
int32_t lbm_batch_step(lbm_batch* batch, const int64_t* nsteps);  /* LBM_ERR_INVALID if a member's force depends on time */
/* The same with each member's time: step j of member k runs at physical time (t0[k] + j) dt[k],
 * as lbm_step(member k, nsteps[k], t0[k], dt[k]) would (the loop's collide!(model, time = t * Δt),
 * src/lattice_boltzmann_model.jl:64-67).  Needed when a member has a time-dependent force
 * (LBM_FORCE_SHEAR, decaying_shear_flow.jl:132-147). */
int32_t lbm_batch_step_timed(lbm_batch* batch, const int64_t* nsteps, const int64_t* t0, const double* dt);
int32_t lbm_batch_set_stream(lbm_batch* batch, void* stream);
int32_t lbm_batch_synchronize(lbm_batch* batch);
int64_t lbm_batch_last_launch_count(const lbm_batch* batch);
const char* lbm_batch_last_error(const lbm_batch* batch);
/* The stop criteria's reductions for many members at once (the per-member next! checks of a
 * sweep, stopping_criteria.jl:17-115): kind LBM_REDUCE_MEAN_VELOCITY, _VELOCITY_CONVERGENCE or
 * _CONSERVED over the members with select[k] != 0 (select NULL: all); out holds count x 16
 * doubles, row k being what lbm_reduce(member k, kind) returns (zeros for members not selected;
 * CONSERVED: row k[3] counts non-finite populations instead of failing).  Synchronous. */
int32_t lbm_batch_reduce(lbm_batch* batch, int32_t kind, const uint8_t* select, double* out);
/* The error norms with analytic fields (LBM_REDUCE_TRACK_ERRORS, _COMPARE) of the selected members
 * at once, e.g. the final TrackHydrodynamicErrors rows of a sweep (track_hydrodynamic_errors.jl:52-242):
 * analytic[k] is member k's lbm_analytic with host planes, as lbm_reduce takes it (entries of
 * members not selected are not read); out as for lbm_batch_reduce.  Synchronous. */
int32_t lbm_batch_reduce_fields(lbm_batch* batch, int32_t kind, const uint8_t* select, const lbm_analytic* analytic,
                                double* out);
/* Block-resident stepping of small members (no counterpart in the reference, which steps each
 * lattice in its own `simulate`).  Per velocity set q (lbm_quadrature index):
 *   resident_max_nodes[q]  members of at most this many nodes take ALL their steps of a
 *                          lbm_batch_step(_timed) call in one kernel launch, their populations held
 *                          in shared memory (0: never; such members use the graph path);
 *   nodes_per_block[q]     nodes per CTA: a resident member runs on a thread-block cluster of
 *                          ceil(n / nodes_per_block[q]) CTAs, rounded up to a power of two, at
 *                          most 8, the pull crossing CTAs through distributed shared memory;
 *   split[q]               warps sharing each node's collision: 1, 2 or 4 (SRT / TRT with FP64 or
 *                          float-float storage from D2Q9 up; 0 and other cases mean 1).
 * A member whose share of both population buffers would not fit one CTA's shared memory takes the
 * graph path.  Results are the same bits on either path (same populations, same collision
 * arithmetic).  lbm_batch_set_schedule(batch, NULL) puts every member on the graph path, the
 * state of a new batch.  The Python binding sets a schedule measured on the GPU. */
typedef struct {
  int64_t resident_max_nodes[7];
  int32_t nodes_per_block[7];
  int32_t split[7];
} lbm_batch_schedule;
int32_t lbm_batch_set_schedule(lbm_batch* batch, const lbm_batch_schedule* schedule);
/* Members issue their own calls on the batch's stream until the batch is destroyed (no ordering
 * between streams per batch call; members must outlive the batch). */
int32_t lbm_batch_share_stream(lbm_batch* batch);

/* ---- adjoint (reverse-mode gradients) -----------------------------------------------------
 * No differentiation exists in the reference; this is the discrete adjoint of the fused step
 * for D2Q9 / D2Q13 lattices with SRT, TRT or regularised MRT, a uniform force and the context's boundary
 * conditions (bounce-back on any side, moving wall: the pull's transpose swaps opposite
 * populations at the walls), FP64 or FP32-deviation storage.  For the loss
 *   L = Σ_x |u(f_T) - u*|²,  f_0 = f_eq(ρ = 1, u0),  f_{t+1} = apply!(stream(collide(f_t))),  T = nsteps,
 * lbm_adjoint_run returns result[0] = L, result[1] = ∂L/∂τ_s (SRT: dL/dτ; MRT: dL/dτ_2, the
 * second-order relaxation time, which also scales the force shift, mrt.jl:91-95; the only one a
 * second-order set's output depends on), result[2] = ∂L/∂τ_a (TRT; 0 for SRT and MRT),
 * result[3..4] = ∂L/∂F, and, if grad_u0 is not NULL, ∂L/∂u0 as two planes of
 * nx*ny (Julia layout, like u0 and u_target).  Memory is bounded by binomial checkpointing
 * (Griewank's schedule): `slots` lattice states are kept (0 selects the fewest with which no
 * forward step is recomputed more than twice), and the reverse sweep recomputes the states it
 * needs from them; with s slots and r = the least count such that C(s + r, s) >= nsteps, no step
 * is recomputed more than r times.  The whole forward + reverse sweep is one CUDA graph.  Loss and
 * parameter sums are FP64, in a fixed order. */
typedef struct lbm_adjoint lbm_adjoint;
int32_t lbm_adjoint_create(lbm_adjoint** adjoint, lbm_ctx* ctx, int64_t nsteps, int64_t slots);
/* The schedule's checkpoint slots, its forward steps (nsteps without checkpointing) and the device
 * memory the adjoint holds, in bytes (any pointer may be NULL). */
int32_t lbm_adjoint_info(const lbm_adjoint* adjoint, int64_t* slots, int64_t* forward_steps, int64_t* device_bytes);
void lbm_adjoint_destroy(lbm_adjoint* adjoint);
int32_t lbm_adjoint_run(lbm_adjoint* adjoint, const double* u0, const double* u_target, double* result,
                        double* grad_u0);
const char* lbm_adjoint_last_error(const lbm_adjoint* adjoint);

/* ---- reductions without allocation --------------------------------------------------------
 * No counterpart in the reference: an addition for callers that cannot allocate device memory
 * -- code running while a CUDA graph is being captured, inside another library's stream
 * callback, or in a host whose device memory belongs to a pool it may not grow -- and that
 * already hold the populations on the device.  lbm_reduce needs a context, and creating one
 * allocates; this entry point allocates nothing (no cudaMalloc, cudaFree or allocating
 * library call).
 *
 * It computes the same sums as lbm_reduce for kind TRACK_ERRORS (out[0..15]), COMPARE
 * (out[0..11]), MEAN_VELOCITY (out[0..1]) or CONSERVED (out[0..3]); other kinds return
 * LBM_ERR_UNSUPPORTED.  Caller-owned inputs and outputs:
 *   f         device array of nx*ny*Q doubles, Julia layout, the observed state (f_stream)
 *   weights   host array of the Q weights, read during the call
 *   analytic  for TRACK_ERRORS / COMPARE: device pointers (on_device = 1) to the analytic fields
 *   out       device array of at least 16 doubles, written asynchronously on `stream`
 *   stream    a cudaStream_t, or NULL for the default stream
 * Scratch: one partial sum per block (at most 608 blocks x 16 sums) in a fixed 77,824-byte
 * static device array, held by every GPU that loads the library until the process exits.  Any
 * lattice below 2^31 nodes fits (larger ones are rejected with LBM_ERR_INVALID), because the
 * grid never exceeds 608 blocks.  Every call reuses that array and keeps the previous call's
 * partial sums in it; a call writes every slot it reads, so nothing needs clearing -- but calls
 * that overlap on the GPU (different streams, or different host threads on one device) race on
 * it: serialise them.  The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress) with that device current; make that first call before any stream
 * capture.  The cached address does not survive cudaDeviceReset: do not call this entry point
 * again in a process that reset the device.  It runs on the calling thread's current device: f,
 * out and the analytic fields must be memory of that device (or managed memory), else
 * LBM_ERR_INVALID.  Returns LBM_OK after the launch; read `out` after synchronising `stream`. */
int32_t lbm_reduce_noalloc(int32_t quadrature, const double* weights, double speed_of_sound_squared, int64_t nx,
                           int64_t ny, const double* f, int32_t kind, const lbm_analytic* analytic, double* out,
                           void* stream);

#ifdef __cplusplus
}
#endif

#endif /* LBM_GB300_H */
