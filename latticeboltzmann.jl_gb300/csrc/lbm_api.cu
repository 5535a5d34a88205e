// lbm_api.cu -- the C ABI of liblbm_gb300.so (declared in include/lbm_gb300.h).
//
// A context holds what LatticeBoltzmannModel holds in the reference
// (src/lattice_boltzmann_model.jl:1-33): the two population arrays (here device buffers in
// the chosen storage), the quadrature, the collision model and the BC list, plus the stream
// the work is issued on.  The device state is either the reference's `f_stream` (after an
// upload) or the post-collision array of the last step, from which `f_stream` is pulled on
// demand; see lbm_step.cuh.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "lbm_ops.cuh"
#include "lbm_resident.cuh"
#include "lbm_adjoint.cuh"

using namespace lbm;

namespace lbm {
cudaError_t batch_launch(int storage, int coll, int qid, const void* statics, const BatchDyn* dyn, int nactive,
                         long long blocks, long long t, cudaStream_t s);
cudaError_t batch_reduce_launch(int storage, int qid, int K, const void* statics, const ReduceArgs* args,
                                const BatchDyn* dyn, int nmem, long long blocks, double* partial, long long part_base,
                                double* out, cudaStream_t s);
size_t batch_static_size(int storage);
cudaError_t resident_launch(int storage, int coll, int qid, const void* statics, const ResidentDyn* dyn, int nmem,
                            int csize, int stride, int threads, int parts, size_t smem_min, cudaStream_t s);
struct AdjArgs;
cudaError_t adj_launch(int op, int qid, int storage, int coll, const void* params, AdjArgs a, const void* src, int pull,
                       const void* lam_next, void* lam_out, double* slots, int nblocks, const double* u0,
                       const double* ut, double* grad, cudaStream_t s);
cudaError_t adj_finish(const double* slots, int nblocks, int k, double* out, cudaStream_t s);
}  // namespace lbm

namespace {

enum Phase { POST_STREAM = 0, POST_COLLIDE = 1 };

typedef cudaError_t (*RunFn)(const OpArgs&);
const RunFn kRun[7] = {run_op_q4, run_op_q5, run_op_q9, run_op_q13, run_op_q17, run_op_q21, run_op_q37};

struct HostLattice {
  int Q, R;
  int cx[LBM_MAX_Q], cy[LBM_MAX_Q], opp[LBM_MAX_Q];
};

template <class L>
HostLattice host_lattice() {
  HostLattice h{};
  h.Q = L::Q;
  h.R = L::R;
  for (int i = 0; i < L::Q; ++i) {
    h.cx[i] = L::cx(i);
    h.cy[i] = L::cy(i);
    h.opp[i] = L::opp(i);
  }
  return h;
}

HostLattice lattice_of(int q) {
  switch (q) {
    case LBM_D2Q4: return host_lattice<D2Q4>();
    case LBM_D2Q5: return host_lattice<D2Q5>();
    case LBM_D2Q9: return host_lattice<D2Q9>();
    case LBM_D2Q13: return host_lattice<D2Q13>();
    case LBM_D2Q17: return host_lattice<D2Q17>();
    case LBM_D2Q21: return host_lattice<D2Q21>();
    default: return host_lattice<D2Q37>();
  }
}

constexpr int kGraphSteps = 64;                  // steps per captured graph (even: parity kept)
constexpr size_t kGraphMaxBytes = 256ull << 20;  // capture only lattices whose step is launch-bound

}  // namespace

struct lbm_ctx {
  int device = 0;
  int qid = 0, Q = 0, R = 1, storage = 0, coll = 0, force_kind = 0;
  int64_t nx = 0, ny = 0, n = 0;
  size_t elem = 8;
  HostLattice lat{};
  void* buf[2] = {nullptr, nullptr};
  int cur = 0;
  int phase = POST_STREAM;
  bool have_state = false;
  cudaStream_t own_stream = nullptr, stream = nullptr;
  StepParams<double> pd{};
  StepParams<float> pf{};
  StepParams<dd> px{};
  ReduceArgs red{};
  double* d_force = nullptr;
  double* d_xr = nullptr;
  double* d_yr = nullptr;
  void* d_nonlinear = nullptr;
  double* d_stage = nullptr;    // FP64 planes for deviation-storage transfers
  double* d_partial = nullptr;  // reduction partial sums
  int red_blocks = 0;
  double* d_out = nullptr;
  double* h_out = nullptr;      // pinned
  double* d_uold = nullptr;
  double* d_analytic = nullptr;
  double* d_macro = nullptr;
  cudaGraphExec_t graph[2] = {nullptr, nullptr};
  // time-dependent force inside graphs: {t0, bits of Δt} on the device (the graphs' steps read it
  // and their last node advances t0), its pinned staging copy and the event of the last upload
  long long* d_time = nullptr;
  long long* h_time = nullptr;
  cudaEvent_t time_ev = nullptr;
  int64_t last_launches = 0;
  std::string err;
};

// The last node of a graph of steps with a time-dependent force: the next launch starts kGraphSteps
// steps later.
__global__ void advance_time_kernel(long long* time, int steps) { time[0] += steps; }

namespace {

// A runtime call that failed (an allocation, a copy, a launch) stays the thread's last CUDA error
// until something reads it.  Once a failure is returned as a status it is read and dropped here,
// so that the launch check of a later, unrelated call (cudaGetLastError after its launches) does
// not report it again.  An error that corrupts the context is not dropped by this: every later
// call returns it.
void drop_reported_error() { (void)cudaGetLastError(); }
// Only the statuses that report a failed CUDA call (an allocation, a copy, a launch) read and drop
// the thread's last CUDA error; a validation failure leaves an error that the caller's own CUDA
// code left pending for the caller to see.
void drop_if_cuda(int status) {
  if (status == LBM_ERR_CUDA || status == LBM_ERR_NOMEM) drop_reported_error();
}

// Makes a context's device current for the scope of an entry point and makes the caller's device
// current again on every return, so that a call on a context of device k leaves the calling
// thread's current device as it found it.
struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    if (cudaGetDevice(&prev) != cudaSuccess) {
      prev = -1;
      drop_reported_error();
    }
    if (prev != dev) cudaSetDevice(dev);
  }
  ~DeviceGuard() {
    int cur = -1;
    if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
  }
  DeviceGuard(const DeviceGuard&) = delete;
  DeviceGuard& operator=(const DeviceGuard&) = delete;
};

// Allocations that leave the pointer null when they fail, so that a destroy after a partial
// creation frees only what was allocated.
template <class T>
bool dev_malloc(T** p, size_t bytes) {
  if (cudaMalloc((void**)p, bytes) == cudaSuccess) return true;
  *p = nullptr;
  return false;
}
template <class T>
bool host_malloc(T** p, size_t bytes) {
  if (cudaMallocHost((void**)p, bytes) == cudaSuccess) return true;
  *p = nullptr;
  return false;
}
bool make_stream(cudaStream_t* st) {
  if (cudaStreamCreateWithFlags(st, cudaStreamNonBlocking) == cudaSuccess) return true;
  *st = nullptr;
  return false;
}
bool make_event(cudaEvent_t* ev) {
  if (cudaEventCreateWithFlags(ev, cudaEventDisableTiming) == cudaSuccess) return true;
  *ev = nullptr;
  return false;
}

int fail(lbm_ctx* c, int status, const std::string& msg) {
  if (c) c->err = msg;
  drop_if_cuda(status);
  return status;
}

int cuda_fail(lbm_ctx* c, cudaError_t e, const char* what) {
  std::string m = std::string(what) + ": " + cudaGetErrorString(e);
  return fail(c, LBM_ERR_CUDA, m);
}

#define LBM_CUDA(ctx, call)                                   \
  do {                                                        \
    cudaError_t e_ = (call);                                  \
    if (e_ != cudaSuccess) return cuda_fail((ctx), e_, #call); \
  } while (0)

OpArgs base_args(lbm_ctx* c, int op) {
  OpArgs a;
  a.op = op;
  a.storage = c->storage;
  a.coll = c->coll;
  a.pd = &c->pd;
  a.pf = &c->pf;
  a.px = &c->px;
  a.red = &c->red;
  a.stream = c->stream;
  return a;
}

int run(lbm_ctx* c, const OpArgs& a) {
  cudaError_t e = kRun[c->qid](a);
  if (e != cudaSuccess) return cuda_fail(c, e, "kernel launch");
  c->last_launches += 1;
  return LBM_OK;
}

// The physical time of the next eagerly launched step, and its time index (the counter of the
// stochastic rounding of SR storage).
void set_time(lbm_ctx* c, double t, int64_t index = 0) {
  c->pd.time = t;
  c->pf.time = t;
  c->px.time = t;
  c->pd.step_index = index;
  c->pf.step_index = index;
  c->px.step_index = index;
}

// Steps captured into a graph take their time index from the device ({t0, Δt} in c->d_time): for
// a time-dependent force, and for stochastically rounded storage (its rounding counter).
bool graph_time(const lbm_ctx* c) {
  return c->force_kind == LBM_FORCE_SHEAR || c->storage == LBM_STORE_F32_DEV_SR;
}

// Steps captured into a graph read their time from the device: step k of the graph runs at
// (t0 + k) Δt with {t0, Δt} in c->d_time (base == nullptr: back to the host-set time).
void set_graph_time(lbm_ctx* c, const long long* base, int k) {
  c->pd.time_base = base;
  c->pf.time_base = base;
  c->px.time_base = base;
  c->pd.time_step = k;
  c->pf.time_step = k;
  c->px.time_step = k;
}

int ensure(lbm_ctx* c, double** p, size_t bytes) {
  if (*p) return LBM_OK;
  cudaError_t e = cudaMalloc((void**)p, bytes);
  if (e != cudaSuccess) {
    *p = nullptr;
    return fail(c, LBM_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  }
  return LBM_OK;
}

// One time step from the current state into the other buffer.
int step_once(lbm_ctx* c) {
  OpArgs a = base_args(c, c->phase == POST_STREAM ? OP_COLLIDE : OP_FUSED);
  a.src = c->buf[c->cur];
  a.dst = c->buf[1 - c->cur];
  int rc = run(c, a);
  if (rc) return rc;
  c->cur ^= 1;
  c->phase = POST_COLLIDE;
  return LBM_OK;
}

// f_stream into the other buffer (pull + BCs), leaving the state POST_STREAM.
int materialise(lbm_ctx* c) {
  if (c->phase == POST_STREAM) return LBM_OK;
  OpArgs a = base_args(c, OP_STREAM_BC);
  a.src = c->buf[c->cur];
  a.dst = c->buf[1 - c->cur];
  int rc = run(c, a);
  if (rc) return rc;
  c->cur ^= 1;
  c->phase = POST_STREAM;
  return LBM_OK;
}

int graph_for_parity(lbm_ctx* c, int parity, cudaGraphExec_t* out) {
  if (c->graph[parity]) {
    *out = c->graph[parity];
    return LBM_OK;
  }
  const bool timed = graph_time(c);
  if (timed && !(c->d_time && c->h_time && c->time_ev)) {  // each part made once, kept if a later one fails
    if ((!c->d_time && !dev_malloc(&c->d_time, 2 * sizeof(long long))) ||
        (!c->h_time && !host_malloc(&c->h_time, 2 * sizeof(long long))))
      return fail(c, LBM_ERR_NOMEM, "time slot of the step graphs");
    if (!c->time_ev && !make_event(&c->time_ev)) return fail(c, LBM_ERR_CUDA, "time event of the step graphs");
  }
  const int saved_cur = c->cur, saved_phase = c->phase;
  const int64_t saved_launches = c->last_launches;
  c->cur = parity;
  c->phase = POST_COLLIDE;
  cudaGraph_t g = nullptr;
  LBM_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  int rc = LBM_OK;
  for (int k = 0; k < kGraphSteps && rc == LBM_OK; ++k) {
    if (timed) set_graph_time(c, c->d_time, k);
    rc = step_once(c);
  }
  if (timed) {
    set_graph_time(c, nullptr, 0);
    if (rc == LBM_OK) {
      advance_time_kernel<<<1, 1, 0, c->stream>>>(c->d_time, kGraphSteps);
      if (cudaGetLastError() != cudaSuccess) rc = fail(c, LBM_ERR_CUDA, "time advance launch");
    }
  }
  cudaError_t e = cudaStreamEndCapture(c->stream, &g);
  c->cur = saved_cur;
  c->phase = saved_phase;
  c->last_launches = saved_launches;
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return cuda_fail(c, e, "cudaStreamEndCapture");
  e = cudaGraphInstantiate(&c->graph[parity], g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    c->graph[parity] = nullptr;
    return cuda_fail(c, e, "cudaGraphInstantiate");
  }
  *out = c->graph[parity];
  return LBM_OK;
}

void free_graphs(lbm_ctx* c) {
  for (int k = 0; k < 2; ++k)
    if (c->graph[k]) {
      cudaGraphExecDestroy(c->graph[k]);
      c->graph[k] = nullptr;
    }
}

int red_kind_k(int kind) {
  switch (kind) {
    case LBM_REDUCE_TRACK_ERRORS: return 16;
    case LBM_REDUCE_COMPARE: return 12;
    case LBM_REDUCE_MEAN_VELOCITY: return 2;
    case LBM_REDUCE_VELOCITY_CONVERGENCE: return 3;
    case LBM_REDUCE_CONSERVED: return 4;
    default: return 0;
  }
}

}  // namespace

extern "C" {

int32_t lbm_abi_version(void) { return LBM_ABI_VERSION; }

const char* lbm_status_string(int32_t s) {
  switch (s) {
    case LBM_OK: return "ok";
    case LBM_ERR_INVALID: return "invalid argument";
    case LBM_ERR_CUDA: return "CUDA error";
    case LBM_ERR_NOMEM: return "out of memory";
    case LBM_ERR_UNSUPPORTED: return "unsupported";
    case LBM_ERR_STATE: return "invalid state";
    case LBM_ERR_NONFINITE: return "non-finite value";
    default: return "unknown status";
  }
}

const char* lbm_last_error(const lbm_ctx* c) { return c ? c->err.c_str() : "null context"; }

int64_t lbm_last_launch_count(const lbm_ctx* c) { return c ? c->last_launches : 0; }

int32_t lbm_create(lbm_ctx** out, const lbm_desc* d) {
  if (!out || !d) return LBM_ERR_INVALID;
  *out = nullptr;
  if (d->quadrature < 0 || d->quadrature > 6) return LBM_ERR_INVALID;
  // each factor is bounded before the product is formed, so the product cannot wrap
  if (d->nx < 1 || d->ny < 1 || d->nx >= (int64_t(1) << 31) || d->ny >= (int64_t(1) << 31) ||
      d->nx * d->ny >= (int64_t(1) << 31))
    return LBM_ERR_INVALID;
  if (d->storage < 0 || d->storage > 5) return LBM_ERR_INVALID;
  if (d->collision < 0 || d->collision > 3) return LBM_ERR_INVALID;
  if (d->force_kind < 0 || d->force_kind > 3) return LBM_ERR_INVALID;
  if (d->nbc < 0 || d->nbc > LBM_MAX_BC || (d->nbc > 0 && !d->bcs)) return LBM_ERR_INVALID;
  if (d->force_kind == LBM_FORCE_FIELD && !d->force_field) return LBM_ERR_INVALID;
  if (d->force_kind == LBM_FORCE_SHEAR && (!d->x_coords || !d->y_coords)) return LBM_ERR_INVALID;
  if (d->collision == LBM_ITERATIVE_INIT && !d->nonlinear) return LBM_ERR_INVALID;

  lbm_ctx* c = new lbm_ctx();
  cudaGetDevice(&c->device);
  c->qid = d->quadrature;
  c->lat = lattice_of(c->qid);
  c->Q = c->lat.Q;
  c->R = c->lat.R;
  c->storage = d->storage;
  c->coll = d->collision;
  c->force_kind = d->force_kind;
  c->nx = d->nx;
  c->ny = d->ny;
  c->n = d->nx * d->ny;
  c->elem = (d->storage == LBM_STORE_F64 || d->storage == LBM_STORE_DF64_DEV || d->storage == LBM_STORE_F64_DD) ? 8
            : (d->storage == LBM_STORE_F32_DEV || d->storage == LBM_STORE_F32_DEV_SR) ? 4 : 2;

  for (int b = 0; b < d->nbc; ++b) {
    const lbm_bc& s = d->bcs[b];
    if (s.kind != LBM_BOUNCE_BACK && s.kind != LBM_MOVING_WALL) { delete c; return LBM_ERR_INVALID; }
    if (s.direction < 0 || s.direction > 3) { delete c; return LBM_ERR_INVALID; }
    if (s.kind == LBM_MOVING_WALL && s.direction != LBM_NORTH) { delete c; return LBM_ERR_UNSUPPORTED; }
    const bool xe = s.x_lo > s.x_hi, ye = s.y_lo > s.y_hi;
    if (s.kind == LBM_BOUNCE_BACK &&
        ((!xe && (s.x_lo < 1 || s.x_hi > d->nx)) || (!ye && (s.y_lo < 1 || s.y_hi > d->ny)))) {
      delete c;
      return LBM_ERR_INVALID;
    }
  }

  // The pair forms give both members of a velocity class {(±a, ±b), (±b, ±a)} one weight (the
  // quadratures of the reference all have this symmetry); other weight tables are rejected.
  for (int i = 0; i < c->Q; ++i)
    for (int j = 0; j < c->Q; ++j) {
      const int ai = std::abs(c->lat.cx[i]), bi = std::abs(c->lat.cy[i]);
      const int aj = std::abs(c->lat.cx[j]), bj = std::abs(c->lat.cy[j]);
      if (std::min(ai, bi) == std::min(aj, bj) && std::max(ai, bi) == std::max(aj, bj) &&
          d->weights[i] != d->weights[j]) {
        delete c;
        return LBM_ERR_INVALID;
      }
    }

  // parameter blocks (FP64 and FP32 copies; the storage selects one)
  StepParams<double>& p = c->pd;
  p.nx = (int)d->nx;
  p.ny = (int)d->ny;
  p.n = c->n;
  for (int s = -3; s <= 3; ++s) {
    p.dxm[s + 3] = (int)(((s % d->nx) + d->nx) % d->nx);
    p.dym[s + 3] = (int)(((s % d->ny) + d->ny) % d->ny);
  }
  for (int i = 0; i < LBM_MAX_Q; ++i) p.w[i] = i < c->Q ? d->weights[i] : 0.0;
  for (int i = 0; i < LBM_MAX_Q; ++i) p.wf[i] = p.w[i];
  p.cs = d->speed_of_sound_squared;
  const double* tau = d->tau;
  if (c->coll == LBM_SRT || c->coll == LBM_ITERATIVE_INIT) {
    p.om_a = 1 - 1 / tau[0];
    p.om_b = 1 / tau[0];
    p.shift = tau[0];
  } else if (c->coll == LBM_TRT) {
    p.inv_ts = 1 / tau[0];
    p.inv_ta = 1 / tau[1];
    p.shift = tau[1];
  } else {
    for (int k = 0; k < 4; ++k) {
      p.mrt_a[k] = 1 - 1 / tau[k];
      p.mrt_b[k] = 1 / tau[k];
    }
    p.shift = tau[1];
  }
  if (c->coll == LBM_SRT || c->coll == LBM_ITERATIVE_INIT) {
    p.pom_s = p.pom_a = 1 / tau[0];
    p.pa_s = p.pa_a = (1 - 1 / tau[0]) / 2;
  } else if (c->coll == LBM_TRT) {
    p.pom_s = 1 / tau[0];
    p.pom_a = 1 / tau[1];
    p.pa_s = (1 - 1 / tau[0]) / 2;
    p.pa_a = (1 - 1 / tau[1]) / 2;
  }
  p.hcs = p.cs / 2;
  p.hcs2 = p.cs * p.cs / 2;
  for (int i = 0; i < LBM_MAX_Q; ++i) p.pws[i] = p.pom_s * p.w[i];
  for (int i = 0; i < LBM_MAX_Q; ++i) p.pwa[i] = p.pom_a * p.w[i];
  p.pa_s2 = 2 * p.pa_s;
  p.force_kind = d->force_kind;
  p.F[0] = d->force[0];
  p.F[1] = d->force[1];
  p.sF[0] = p.shift * p.F[0];
  p.sF[1] = p.shift * p.F[1];
  for (int k = 0; k < 6; ++k) p.shear[k] = d->shear[k];
  p.nbc = d->nbc;
  for (int b = 0; b < d->nbc; ++b) {
    const lbm_bc& s = d->bcs[b];
    BCDev& t = p.bc[b];
    t.kind = s.kind;
    t.dir = s.direction;
    t.x_lo = s.x_lo - 1;
    t.x_hi = s.x_hi - 1;
    t.y_lo = s.y_lo - 1;
    t.y_hi = s.y_hi - 1;
    for (int i = 0; i < LBM_MAX_Q; ++i) t.add[i] = 0.0;
    if (s.kind == LBM_MOVING_WALL) {
      // a_1 = w_i * cs * dot(ρ_w u_w, c_i), the added term is 2 a_1 (moving_wall.jl:20-33)
      const double a1x = s.rho * s.u[0], a1y = s.rho * s.u[1];
      for (int i = 0; i < c->Q; ++i) {
        const double a1 = d->weights[i] * d->speed_of_sound_squared *
                          (a1x * (c->lat.cx[i] * 1.0) + a1y * (c->lat.cy[i] * 1.0));
        t.add[i] = 2 * a1;
      }
    }
  }
  // FP32 copy
  StepParams<float>& q = c->pf;
  q.nx = p.nx;
  q.ny = p.ny;
  q.n = p.n;
  for (int k = 0; k < 7; ++k) {
    q.dxm[k] = p.dxm[k];
    q.dym[k] = p.dym[k];
  }
  for (int i = 0; i < LBM_MAX_Q; ++i) q.w[i] = (float)p.w[i];
  for (int i = 0; i < LBM_MAX_Q; ++i) q.wf[i] = p.w[i];
  q.cs = (float)p.cs;
  q.om_a = (float)p.om_a;
  q.om_b = (float)p.om_b;
  q.inv_ts = (float)p.inv_ts;
  q.inv_ta = (float)p.inv_ta;
  q.shift = (float)p.shift;
  q.pa_s = (float)p.pa_s;
  q.pa_a = (float)p.pa_a;
  q.pom_s = (float)p.pom_s;
  q.pom_a = (float)p.pom_a;
  q.hcs = (float)p.hcs;
  q.hcs2 = (float)p.hcs2;
  for (int i = 0; i < LBM_MAX_Q; ++i) q.pws[i] = (float)p.pws[i];
  for (int i = 0; i < LBM_MAX_Q; ++i) q.pwa[i] = (float)p.pwa[i];
  q.pa_s2 = (float)p.pa_s2;
  q.sF[0] = (float)p.sF[0];
  q.sF[1] = (float)p.sF[1];
  for (int k = 0; k < 4; ++k) {
    q.mrt_a[k] = (float)p.mrt_a[k];
    q.mrt_b[k] = (float)p.mrt_b[k];
  }
  q.force_kind = p.force_kind;
  q.F[0] = (float)p.F[0];
  q.F[1] = (float)p.F[1];
  for (int k = 0; k < 6; ++k) q.shear[k] = p.shear[k];
  q.nbc = p.nbc;
  for (int b = 0; b < p.nbc; ++b) q.bc[b] = p.bc[b];
  // First-order equilibrium coefficients of the deviation storages, w1_i = (1/c_s²) w_i.  The
  // equilibrium's momentum is (Σ_i w1_i c_i c_i)·ρu; with w1 rounded to FP32 the second moment is
  // 1 + O(1e-8), and the relaxation turns that into a momentum drift that grows linearly in time.
  // So one velocity class (of nonzero weight) absorbs the rounding: its coefficient is solved
  // from Σ_i w1_i c_ix² = 1 over the already-rounded others, and the class whose solution is
  // representable exactly is preferred (D2Q4/5/9/13: exact; D2Q17/37: residual ~1e-10).
  {
    for (int i = 0; i < LBM_MAX_Q; ++i) p.w1[i] = i < c->Q ? p.cs * p.w[i] : 0.0;
    for (int i = 0; i < LBM_MAX_Q; ++i) p.pw1a[i] = p.pom_a * p.w1[i];
    float w1f[LBM_MAX_Q];
    for (int i = 0; i < LBM_MAX_Q; ++i) w1f[i] = (float)p.w1[i];
    long double best_res = -1.0L;
    float best_val = 0.f;
    int best_cls = -1;
    for (int i = 0; i < c->Q; ++i) {  // candidate class: the velocities with i's (|cx|, |cy|) set
      const int a = std::abs(c->lat.cx[i]), b = std::abs(c->lat.cy[i]);
      const int lo_ab = std::min(a, b), hi_ab = std::max(a, b);
      if (p.w[i] == 0.0) continue;
      long double other = 0.0L, c2 = 0.0L;
      for (int j = 0; j < c->Q; ++j) {
        const int aj = std::abs(c->lat.cx[j]), bj = std::abs(c->lat.cy[j]);
        const long double cx2 = (long double)(c->lat.cx[j] * c->lat.cx[j]);
        if (std::min(aj, bj) == lo_ab && std::max(aj, bj) == hi_ab) c2 += cx2;
        else other += (long double)w1f[j] * cx2;
      }
      if (c2 == 0.0L) continue;
      const float val = (float)((1.0L - other) / c2);
      long double res = 1.0L - other - (long double)val * c2;
      if (res < 0) res = -res;
      if (best_cls < 0 || res < best_res) {
        best_res = res;
        best_val = val;
        best_cls = i;
      }
    }
    if (best_cls >= 0) {
      const int a = std::abs(c->lat.cx[best_cls]), b = std::abs(c->lat.cy[best_cls]);
      for (int j = 0; j < c->Q; ++j) {
        const int aj = std::abs(c->lat.cx[j]), bj = std::abs(c->lat.cy[j]);
        if (std::min(aj, bj) == std::min(a, b) && std::max(aj, bj) == std::max(a, b)) w1f[j] = best_val;
      }
    }
    for (int i = 0; i < LBM_MAX_Q; ++i) q.w1[i] = w1f[i];
    for (int i = 0; i < LBM_MAX_Q; ++i) q.pw1a[i] = (float)p.pom_a * w1f[i];
  }
  // float-float copy (every constant split once on the host)
  StepParams<dd>& x = c->px;
  x.nx = p.nx;
  x.ny = p.ny;
  x.n = p.n;
  for (int k = 0; k < 7; ++k) {
    x.dxm[k] = p.dxm[k];
    x.dym[k] = p.dym[k];
  }
  for (int i = 0; i < LBM_MAX_Q; ++i) x.w[i] = dd(p.w[i]);
  for (int i = 0; i < LBM_MAX_Q; ++i) x.wf[i] = p.w[i];
  for (int i = 0; i < LBM_MAX_Q; ++i) x.w1[i] = dd(p.w1[i]);
  x.cs = dd(p.cs);
  x.om_a = dd(p.om_a);
  x.om_b = dd(p.om_b);
  x.inv_ts = dd(p.inv_ts);
  x.inv_ta = dd(p.inv_ta);
  x.shift = dd(p.shift);
  x.pa_s = dd(p.pa_s);
  x.pa_a = dd(p.pa_a);
  x.pom_s = dd(p.pom_s);
  x.pom_a = dd(p.pom_a);
  x.hcs = dd(p.hcs);
  x.hcs2 = dd(p.hcs2);
  for (int i = 0; i < LBM_MAX_Q; ++i) x.pws[i] = dd(p.pws[i]);
  for (int i = 0; i < LBM_MAX_Q; ++i) x.pwa[i] = dd(p.pwa[i]);
  for (int i = 0; i < LBM_MAX_Q; ++i) x.pw1a[i] = dd(p.pom_a * p.w1[i]);
  x.pa_s2 = dd(p.pa_s2);
  x.sF[0] = dd(p.sF[0]);
  x.sF[1] = dd(p.sF[1]);
  for (int k = 0; k < 4; ++k) {
    x.mrt_a[k] = dd(p.mrt_a[k]);
    x.mrt_b[k] = dd(p.mrt_b[k]);
  }
  x.force_kind = p.force_kind;
  x.F[0] = dd(p.F[0]);
  x.F[1] = dd(p.F[1]);
  for (int k = 0; k < 6; ++k) x.shear[k] = p.shear[k];
  x.nbc = p.nbc;
  for (int b = 0; b < p.nbc; ++b) x.bc[b] = p.bc[b];

  // reduction constants
  for (int i = 0; i < LBM_MAX_Q; ++i) c->red.w[i] = p.w[i];
  c->red.cs = p.cs;
  c->red.q_low_order = (c->qid == LBM_D2Q4 || c->qid == LBM_D2Q5) ? 1 : 0;

  const size_t bytes = (size_t)c->n * c->Q * c->elem;
  for (int k = 0; k < 2; ++k) {
    if (!dev_malloc(&c->buf[k], bytes)) {
      lbm_destroy(c);
      drop_reported_error();
      return LBM_ERR_NOMEM;
    }
  }
  if (!make_stream(&c->own_stream)) {
    lbm_destroy(c);
    drop_reported_error();
    return LBM_ERR_CUDA;
  }
  c->stream = c->own_stream;
  // the reduction scratch (lbm_reduce) is allocated at the first reduction: members of a batch,
  // whose reductions run batched, never need it, and a sweep creates thousands of them
  c->red_blocks = (int)std::min<int64_t>((c->n + kRedThreads - 1) / kRedThreads, kSumBlocks);
  if (d->force_kind == LBM_FORCE_FIELD) {
    if (!dev_malloc(&c->d_force, (size_t)c->n * 2 * sizeof(double)) ||
        cudaMemcpy(c->d_force, d->force_field, (size_t)c->n * 2 * sizeof(double), cudaMemcpyHostToDevice) !=
            cudaSuccess) {
      lbm_destroy(c);
      drop_reported_error();
      return LBM_ERR_NOMEM;
    }
  }
  if (d->force_kind == LBM_FORCE_SHEAR) {
    if (!dev_malloc(&c->d_xr, (size_t)c->nx * sizeof(double)) ||
        !dev_malloc(&c->d_yr, (size_t)c->ny * sizeof(double)) ||
        cudaMemcpy(c->d_xr, d->x_coords, (size_t)c->nx * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(c->d_yr, d->y_coords, (size_t)c->ny * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess) {
      lbm_destroy(c);
      drop_reported_error();
      return LBM_ERR_NOMEM;
    }
  }
  if (c->coll == LBM_ITERATIVE_INIT) {
    const size_t cnt = (size_t)c->n * c->Q;
    if (c->storage == LBM_STORE_F64) {
      if (!dev_malloc(&c->d_nonlinear, cnt * sizeof(double)) ||
          cudaMemcpy(c->d_nonlinear, d->nonlinear, cnt * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess) {
        lbm_destroy(c);
        drop_reported_error();
        return LBM_ERR_NOMEM;
      }
    } else if (c->storage == LBM_STORE_DF64_DEV || c->storage == LBM_STORE_F32_DEV_SR ||
               c->storage == LBM_STORE_F64_DD) {  // float-float arithmetic
      std::vector<dd> tmp(cnt);
      for (size_t k = 0; k < cnt; ++k) tmp[k] = dd(d->nonlinear[k]);
      if (!dev_malloc(&c->d_nonlinear, cnt * sizeof(dd)) ||
          cudaMemcpy(c->d_nonlinear, tmp.data(), cnt * sizeof(dd), cudaMemcpyHostToDevice) != cudaSuccess) {
        lbm_destroy(c);
        drop_reported_error();
        return LBM_ERR_NOMEM;
      }
    } else {
      std::vector<float> tmp(cnt);
      for (size_t k = 0; k < cnt; ++k) tmp[k] = (float)d->nonlinear[k];
      if (!dev_malloc(&c->d_nonlinear, cnt * sizeof(float)) ||
          cudaMemcpy(c->d_nonlinear, tmp.data(), cnt * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess) {
        lbm_destroy(c);
        drop_reported_error();
        return LBM_ERR_NOMEM;
      }
    }
  }
  p.Ffield = q.Ffield = x.Ffield = c->d_force;
  p.xr = q.xr = x.xr = c->d_xr;
  p.yr = q.yr = x.yr = c->d_yr;
  x.nonlinear = static_cast<const dd*>(c->d_nonlinear);
  p.nonlinear = static_cast<const double*>(c->d_nonlinear);
  q.nonlinear = static_cast<const float*>(c->d_nonlinear);
  *out = c;
  return LBM_OK;
}

void lbm_destroy(lbm_ctx* c) {
  if (!c) return;
  DeviceGuard device_guard(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  free_graphs(c);
  for (int k = 0; k < 2; ++k) cudaFree(c->buf[k]);
  cudaFree(c->d_time);
  if (c->h_time) cudaFreeHost(c->h_time);
  if (c->time_ev) cudaEventDestroy(c->time_ev);
  cudaFree(c->d_force);
  cudaFree(c->d_xr);
  cudaFree(c->d_yr);
  cudaFree(c->d_nonlinear);
  cudaFree(c->d_stage);
  cudaFree(c->d_partial);
  cudaFree(c->d_out);
  if (c->h_out) cudaFreeHost(c->h_out);
  cudaFree(c->d_uold);
  cudaFree(c->d_analytic);
  cudaFree(c->d_macro);
  if (c->own_stream) cudaStreamDestroy(c->own_stream);
  delete c;
}

int32_t lbm_set_stream(lbm_ctx* c, void* stream) {
  if (!c) return LBM_ERR_INVALID;
  DeviceGuard device_guard(c->device);
  LBM_CUDA(c, cudaStreamSynchronize(c->stream));
  c->stream = stream ? static_cast<cudaStream_t>(stream) : c->own_stream;
  free_graphs(c);  // graphs are captured on, and launched into, a stream; recapture lazily
  return LBM_OK;
}

int32_t lbm_synchronize(lbm_ctx* c) {
  if (!c) return LBM_ERR_INVALID;
  DeviceGuard device_guard(c->device);
  LBM_CUDA(c, cudaStreamSynchronize(c->stream));
  return LBM_OK;
}

static int upload_impl(lbm_ctx* c, const double* f, cudaMemcpyKind kind) {
  if (!c || !f) return LBM_ERR_INVALID;
  DeviceGuard device_guard(c->device);
  const size_t cnt = (size_t)c->n * c->Q;
  if (c->storage == LBM_STORE_F64) {
    LBM_CUDA(c, cudaMemcpyAsync(c->buf[0], f, cnt * sizeof(double), kind, c->stream));
  } else {
    int rc = ensure(c, &c->d_stage, cnt * sizeof(double));
    if (rc) return rc;
    LBM_CUDA(c, cudaMemcpyAsync(c->d_stage, f, cnt * sizeof(double), kind, c->stream));
    OpArgs a = base_args(c, OP_NARROW);
    a.src = c->d_stage;
    a.dst = c->buf[0];
    rc = run(c, a);
    if (rc) return rc;
  }
  c->cur = 0;
  c->phase = POST_STREAM;
  c->have_state = true;
  LBM_CUDA(c, cudaStreamSynchronize(c->stream));
  return LBM_OK;
}

int32_t lbm_initialize_fields(lbm_ctx* c, const double* rho, const double* ux, const double* uy, const double* T,
                              const double* sxx, const double* sxy, const double* syy, double stress_coef,
                              int32_t stress_times_rho) {
  if (!c) return LBM_ERR_INVALID;
  const bool any_s = sxx || sxy || syy, all_s = sxx && sxy && syy;
  if (any_s && !all_s) return fail(c, LBM_ERR_INVALID, "the stress tensor needs sxx, sxy and syy");
  DeviceGuard device_guard(c->device);
  const double* host[7] = {rho, ux, uy, T, sxx, sxy, syy};
  int nplanes = 0;
  for (const double* h : host) nplanes += h ? 1 : 0;
  double* d = nullptr;
  if (nplanes > 0) {
    cudaError_t e = cudaMalloc((void**)&d, (size_t)c->n * nplanes * sizeof(double));
    if (e != cudaSuccess) return fail(c, LBM_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  }
  const double* dev[7] = {};
  int k = 0;
  for (int j = 0; j < 7; ++j) {
    if (!host[j]) continue;
    double* plane = d + (size_t)k++ * c->n;
    cudaError_t e = cudaMemcpyAsync(plane, host[j], (size_t)c->n * sizeof(double), cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess) {
      cudaFree(d);
      return cuda_fail(c, e, "cudaMemcpyAsync");
    }
    dev[j] = plane;
  }
  InitFields in{dev[0], dev[1], dev[2], dev[3], dev[4], dev[5], dev[6], stress_coef, stress_times_rho ? 1 : 0};
  OpArgs a = base_args(c, OP_INIT_FIELDS);
  a.init = &in;
  a.dst = c->buf[0];
  int rc = run(c, a);
  cudaError_t e = cudaStreamSynchronize(c->stream);
  cudaFree(d);
  if (rc) return rc;
  if (e != cudaSuccess) return cuda_fail(c, e, "initialize");
  c->cur = 0;
  c->phase = POST_STREAM;
  c->have_state = true;
  return LBM_OK;
}

int32_t lbm_upload(lbm_ctx* c, const double* f) { return upload_impl(c, f, cudaMemcpyHostToDevice); }
int32_t lbm_upload_device(lbm_ctx* c, const double* f) { return upload_impl(c, f, cudaMemcpyDeviceToDevice); }

static int download_impl(lbm_ctx* c, double* f, cudaMemcpyKind kind) {
  if (!c || !f) return LBM_ERR_INVALID;
  if (!c->have_state) return fail(c, LBM_ERR_STATE, "no state uploaded");
  DeviceGuard device_guard(c->device);
  const size_t cnt = (size_t)c->n * c->Q;
  if (c->storage == LBM_STORE_F64) {
    int rc = materialise(c);
    if (rc) return rc;
    LBM_CUDA(c, cudaMemcpyAsync(f, c->buf[c->cur], cnt * sizeof(double), kind, c->stream));
  } else {
    int rc = ensure(c, &c->d_stage, cnt * sizeof(double));
    if (rc) return rc;
    OpArgs a = base_args(c, OP_WIDEN);
    a.pull = c->phase == POST_COLLIDE;
    a.src = c->buf[c->cur];
    a.dst = c->d_stage;
    rc = run(c, a);
    if (rc) return rc;
    LBM_CUDA(c, cudaMemcpyAsync(f, c->d_stage, cnt * sizeof(double), kind, c->stream));
  }
  LBM_CUDA(c, cudaStreamSynchronize(c->stream));
  return LBM_OK;
}

int32_t lbm_download(lbm_ctx* c, double* f) { return download_impl(c, f, cudaMemcpyDeviceToHost); }
int32_t lbm_download_device(lbm_ctx* c, double* f) { return download_impl(c, f, cudaMemcpyDeviceToDevice); }

int32_t lbm_step(lbm_ctx* c, int64_t nsteps, int64_t t0, double dt) {
  if (!c || nsteps < 0) return LBM_ERR_INVALID;
  if (!c->have_state) return fail(c, LBM_ERR_STATE, "no state uploaded");
  DeviceGuard device_guard(c->device);
  c->last_launches = 0;
  int64_t k = 0;
  const bool time_dependent = graph_time(c);
  const size_t bytes = (size_t)c->n * c->Q * c->elem;
  const bool use_graph = bytes <= kGraphMaxBytes;
  bool time_uploaded = false;  // graphs with device time: {t0 + k, Δt} on the device for them
  while (k < nsteps) {
    set_time(c, (double)(t0 + k) * dt, t0 + k);
    if (use_graph && c->phase == POST_COLLIDE && nsteps - k >= kGraphSteps) {
      cudaGraphExec_t g = nullptr;
      int rc = graph_for_parity(c, c->cur, &g);
      if (rc) return rc;
      if (time_dependent && !time_uploaded) {  // the graphs that follow advance it themselves
        LBM_CUDA(c, cudaEventSynchronize(c->time_ev));  // the staging copy is free again
        c->h_time[0] = (long long)(t0 + k);
        std::memcpy(&c->h_time[1], &dt, sizeof(double));
        LBM_CUDA(c, cudaMemcpyAsync(c->d_time, c->h_time, 2 * sizeof(long long), cudaMemcpyHostToDevice, c->stream));
        LBM_CUDA(c, cudaEventRecord(c->time_ev, c->stream));
        time_uploaded = true;
      }
      LBM_CUDA(c, cudaGraphLaunch(g, c->stream));
      c->last_launches += kGraphSteps + (time_dependent ? 1 : 0);  // + the time advance
      k += kGraphSteps;  // even number of steps: the state returns to the same buffer
      continue;
    }
    int rc = step_once(c);
    if (rc) return rc;
    ++k;
  }
  return LBM_OK;
}

int32_t lbm_reduce(lbm_ctx* c, int32_t kind, const lbm_analytic* an, double* out) {
  if (!c || !out) return LBM_ERR_INVALID;
  if (!c->have_state) return fail(c, LBM_ERR_STATE, "no state uploaded");
  DeviceGuard device_guard(c->device);
  if ((!c->d_partial && !dev_malloc(&c->d_partial, (size_t)c->red_blocks * kRedMaxK * sizeof(double))) ||
      (!c->d_out && !dev_malloc(&c->d_out, kRedMaxK * sizeof(double))) ||
      (!c->h_out && !host_malloc(&c->h_out, kRedMaxK * sizeof(double))))
    return fail(c, LBM_ERR_NOMEM, "reduction scratch");
  const bool pull = c->phase == POST_COLLIDE;
  if (kind == LBM_REDUCE_DENSITY_AT) {
    const int64_t ix = (int64_t)out[0], iy = (int64_t)out[1];
    if (ix < 0 || ix >= c->nx || iy < 0 || iy >= c->ny) return fail(c, LBM_ERR_INVALID, "node out of range");
    OpArgs a = base_args(c, OP_NODE_DENSITY);
    a.pull = pull;
    a.src = c->buf[c->cur];
    a.node_x = (int)ix;
    a.node_y = (int)iy;
    a.out = c->d_out;
    int rc = run(c, a);
    if (rc) return rc;
    LBM_CUDA(c, cudaMemcpyAsync(c->h_out, c->d_out, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    LBM_CUDA(c, cudaStreamSynchronize(c->stream));
    out[0] = c->h_out[0];
    return LBM_OK;
  }
  const int K = red_kind_k(kind);
  if (!K) return fail(c, LBM_ERR_INVALID, "unknown reduction kind");
  ReduceArgs r = c->red;
  r.kind = kind;
  if (kind == LBM_REDUCE_TRACK_ERRORS || kind == LBM_REDUCE_COMPARE) {
    if (!an) return fail(c, LBM_ERR_INVALID, "analytic fields required");
    const double* src[8] = {an->rho, an->ux, an->uy, an->p, an->sxx, an->syx, an->sxy, an->syy};
    const int need = kind == LBM_REDUCE_TRACK_ERRORS ? 8 : 4;
    for (int k = 0; k < need; ++k)
      if (!src[k]) return fail(c, LBM_ERR_INVALID, "missing analytic field");
    const double* dptr[8];
    if (an->on_device) {
      for (int k = 0; k < 8; ++k) dptr[k] = src[k];
    } else {
      int rc = ensure(c, &c->d_analytic, (size_t)c->n * 8 * sizeof(double));
      if (rc) return rc;
      bool one_block = true;  // the eight planes consecutive in one host array: one copy
      for (int k = 0; k < 8; ++k) one_block = one_block && src[k] == src[0] + (size_t)k * c->n;
      for (int k = 0; k < 8; ++k) dptr[k] = c->d_analytic + (size_t)k * c->n;
      if (one_block) {
        LBM_CUDA(c, cudaMemcpyAsync(c->d_analytic, src[0], (size_t)c->n * 8 * sizeof(double), cudaMemcpyHostToDevice,
                                    c->stream));
      } else {
        for (int k = 0; k < 8; ++k)
          if (src[k])
            LBM_CUDA(c, cudaMemcpyAsync((void*)dptr[k], src[k], (size_t)c->n * sizeof(double), cudaMemcpyHostToDevice,
                                        c->stream));
      }
    }
    r.rho_a = dptr[0];
    r.ux_a = dptr[1];
    r.uy_a = dptr[2];
    r.p_a = dptr[3];
    r.sxx_a = dptr[4];
    r.syx_a = dptr[5];
    r.sxy_a = dptr[6];
    r.syy_a = dptr[7];
    r.tau = an->tau;
    r.u_max = an->u_max;
    r.area = an->area;
  }
  if (kind == LBM_REDUCE_VELOCITY_CONVERGENCE) {
    if (!c->d_uold) {
      int rc = ensure(c, &c->d_uold, (size_t)c->n * 2 * sizeof(double));
      if (rc) return rc;
      LBM_CUDA(c, cudaMemsetAsync(c->d_uold, 0, (size_t)c->n * 2 * sizeof(double), c->stream));
    }
    r.u_old = c->d_uold;
  }
  OpArgs a = base_args(c, OP_REDUCE);
  a.red = &r;
  a.red_k = K;
  a.pull = pull;
  a.src = c->buf[c->cur];
  a.partial = c->d_partial;
  a.nblocks = c->red_blocks;
  a.out = c->d_out;
  int rc = run(c, a);
  if (rc) return rc;
  LBM_CUDA(c, cudaMemcpyAsync(c->h_out, c->d_out, K * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  LBM_CUDA(c, cudaStreamSynchronize(c->stream));
  for (int k = 0; k < K; ++k) out[k] = c->h_out[k];
  if (kind == LBM_REDUCE_CONSERVED && out[3] != 0.0) return fail(c, LBM_ERR_NONFINITE, "non-finite populations");
  return LBM_OK;
}

int32_t lbm_macroscopic(lbm_ctx* c, double* rho, double* ux, double* uy) {
  if (!c) return LBM_ERR_INVALID;
  if (!c->have_state) return fail(c, LBM_ERR_STATE, "no state uploaded");
  DeviceGuard device_guard(c->device);
  int rc = ensure(c, &c->d_macro, (size_t)c->n * 3 * sizeof(double));
  if (rc) return rc;
  OpArgs a = base_args(c, OP_MACRO);
  a.pull = c->phase == POST_COLLIDE;
  a.src = c->buf[c->cur];
  a.dst = c->d_macro;
  rc = run(c, a);
  if (rc) return rc;
  double* outs[3] = {rho, ux, uy};
  for (int k = 0; k < 3; ++k)
    if (outs[k])
      LBM_CUDA(c, cudaMemcpyAsync(outs[k], c->d_macro + (size_t)k * c->n, (size_t)c->n * sizeof(double),
                                  cudaMemcpyDeviceToHost, c->stream));
  LBM_CUDA(c, cudaStreamSynchronize(c->stream));
  return LBM_OK;
}

int32_t lbm_collide_device(lbm_ctx* c, const double* f_in, double* f_out, double time) {
  if (!c || !f_in || !f_out) return LBM_ERR_INVALID;
  if (c->storage != LBM_STORE_F64) return fail(c, LBM_ERR_UNSUPPORTED, "device operators need FP64 storage");
  DeviceGuard device_guard(c->device);
  set_time(c, time);
  OpArgs a = base_args(c, OP_COLLIDE);
  a.src = f_in;
  a.dst = f_out;
  return run(c, a);
}

int32_t lbm_stream_device(lbm_ctx* c, const double* f, double* f_new) {
  if (!c || !f || !f_new) return LBM_ERR_INVALID;
  if (c->storage != LBM_STORE_F64) return fail(c, LBM_ERR_UNSUPPORTED, "device operators need FP64 storage");
  DeviceGuard device_guard(c->device);
  OpArgs a = base_args(c, OP_STREAM);
  a.src = f;
  a.dst = f_new;
  return run(c, a);
}

int32_t lbm_apply_bcs_device(lbm_ctx* c, double* f_new, const double* f_old) {
  if (!c || !f_new || !f_old) return LBM_ERR_INVALID;
  if (c->storage != LBM_STORE_F64) return fail(c, LBM_ERR_UNSUPPORTED, "device operators need FP64 storage");
  DeviceGuard device_guard(c->device);
  if (c->pd.nbc == 0) return LBM_OK;
  OpArgs a = base_args(c, OP_APPLY_BC);
  a.src = f_old;
  a.dst = f_new;
  return run(c, a);
}


}  // extern "C"

// ---- batches -------------------------------------------------------------------------------

struct lbm_batch {
  std::vector<lbm_ctx*> members;
  int device = 0, storage = 0, coll = 0;
  cudaStream_t own_stream = nullptr, stream = nullptr;
  void* d_static = nullptr;       // BatchStatic<CT> per member, uploaded once
  BatchDyn* d_dyn = nullptr;      // per call, launch order
  BatchDyn* h_dyn = nullptr;      // pinned staging copy
  cudaEvent_t staged = nullptr;   // the last upload from h_dyn has completed
  // block-resident members (lbm_resident.cuh): the schedule, the per-call descriptors (staged
  // with h_dyn) and one stream + event per resident launch, forked from and joined to `stream`
  lbm_batch_schedule schedule{};  // zero: every member on the graph path
  ResidentDyn* d_rdyn = nullptr;
  ResidentDyn* h_rdyn = nullptr;
  std::vector<cudaStream_t> res_streams;
  std::vector<cudaEvent_t> res_events;
  cudaEvent_t res_fork = nullptr;
  int64_t res_launches = 0;
  int sm_count = 0;                // the device's SMs and shared memory per SM (bytes)
  int smem_per_sm = 0;
  ReduceArgs* d_rargs = nullptr;  // per member, set up by the first reduction
  std::vector<ReduceArgs> h_rargs; // host copy of the same
  ReduceArgs* d_rargs_call = nullptr;  // per member, with this call's analytic fields
  double* h_ranal = nullptr;       // pinned staging of the analytic planes
  double* d_ranal = nullptr;
  size_t ranal_cap = 0;            // doubles
  double* d_rpartial = nullptr;
  long long rpartial_blocks = 0;
  double* d_rout = nullptr;       // count x kRedMaxK
  double* h_rout = nullptr;       // pinned
  cudaEvent_t done = nullptr;
  cudaGraphExec_t graph = nullptr;
  std::vector<int64_t> graph_key;  // sorted step counts the graph was captured for
  std::vector<int> graph_order;
  int64_t graph_launches = 0;
  int64_t last_launches = 0;
  bool shared = false;             // the members issue their own work on the batch's stream
  bool time_dependent = false;     // a member's force depends on time (its steps need their times)
  // per velocity-set group: a stream and an event, so that the groups' step chains are
  // independent branches of the batch graph (created with the first multi-group graph)
  std::vector<cudaStream_t> group_streams;
  std::vector<cudaEvent_t> group_events;
  cudaEvent_t fork = nullptr;
  std::string err;
};

namespace {

int bfail(lbm_batch* b, int status, const std::string& msg) {
  if (b) b->err = msg;
  drop_if_cuda(status);
  return status;
}

template <class CT>
void fill_static(BatchStatic<CT>& m, const StepParams<CT>& p, const lbm_ctx* c) {
  m.p = p;
  m.buf0 = c->buf[0];
  m.buf1 = c->buf[1];
}

// The batch stream waits for the members' own streams (uploads and reductions issued there),
// once per distinct stream.
int batch_wait_members(lbm_batch* b) {
  std::vector<cudaStream_t> seen;
  for (lbm_ctx* c : b->members) {
    if (c->stream == b->stream || std::find(seen.begin(), seen.end(), c->stream) != seen.end()) continue;
    seen.push_back(c->stream);
    if (cudaEventRecord(b->done, c->stream) != cudaSuccess || cudaStreamWaitEvent(b->stream, b->done, 0) != cudaSuccess)
      return bfail(b, LBM_ERR_CUDA, "ordering member streams");
  }
  return LBM_OK;
}

// The members' streams wait for the batch's work, once per distinct stream.
int batch_release_members(lbm_batch* b) {
  if (cudaEventRecord(b->done, b->stream) != cudaSuccess) return bfail(b, LBM_ERR_CUDA, "event");
  std::vector<cudaStream_t> seen;
  for (lbm_ctx* c : b->members) {
    if (c->stream == b->stream || std::find(seen.begin(), seen.end(), c->stream) != seen.end()) continue;
    seen.push_back(c->stream);
    if (cudaStreamWaitEvent(c->stream, b->done, 0) != cudaSuccess) return bfail(b, LBM_ERR_CUDA, "member wait");
  }
  return LBM_OK;
}

// Uploads dyn[0..count) through the pinned staging buffer (waiting for the previous upload from
// it to finish before it is overwritten).
int batch_upload_dyn(lbm_batch* b, const std::vector<BatchDyn>& dyn, const std::vector<ResidentDyn>& rdyn) {
  if (cudaEventSynchronize(b->staged) != cudaSuccess) return bfail(b, LBM_ERR_CUDA, "staging wait");
  std::copy(dyn.begin(), dyn.end(), b->h_dyn);
  std::copy(rdyn.begin(), rdyn.end(), b->h_rdyn);
  if (cudaMemcpyAsync(b->d_dyn, b->h_dyn, sizeof(BatchDyn) * dyn.size(), cudaMemcpyHostToDevice, b->stream) !=
          cudaSuccess ||
      (!rdyn.empty() && cudaMemcpyAsync(b->d_rdyn, b->h_rdyn, sizeof(ResidentDyn) * rdyn.size(),
                                        cudaMemcpyHostToDevice, b->stream) != cudaSuccess) ||
      cudaEventRecord(b->staged, b->stream) != cudaSuccess)
    return bfail(b, LBM_ERR_CUDA, "descriptor upload");
  return LBM_OK;
}

// Bytes of one population (both buffers) of a node in the batch's storage.
size_t storage_bytes(int storage) {
  return storage == LBM_STORE_F32_DEV ? 4 : 8;
}

// The cluster size of a block-resident member of n nodes, or 0 when the member takes the graph
// path: at most resident_max_nodes[q] nodes, ceil(n / nodes_per_block[q]) CTAs rounded up to a
// power of two (at most 8), and both buffers of a CTA's share within one CTA's shared memory.
int resident_cluster(const lbm_batch* b, const lbm_ctx* c) {
  const int64_t lim = b->schedule.resident_max_nodes[c->qid];
  const int per = b->schedule.nodes_per_block[c->qid];
  if (lim <= 0 || per <= 0 || c->n > lim) return 0;
  int csize = 1;
  while (csize < kResidentMaxCluster && (int64_t)csize * per < c->n) csize *= 2;
  const int64_t chunk = (c->n + csize - 1) / csize;
  if (2 * (size_t)c->Q * (size_t)chunk * storage_bytes(b->storage) > kResidentMaxSmem) return 0;
  return csize;
}

// Warps sharing each node's collision in a resident launch (lbm_resident.cuh builds splits for
// SRT / TRT with FP64 or float-float storage from D2Q9 up).
int resident_parts(const lbm_batch* b, const lbm_ctx* c) {
  const int s = b->schedule.split[c->qid];
  if ((s != 2 && s != 4) || (b->coll != LBM_SRT && b->coll != LBM_TRT) || c->Q < 9 ||
      (b->storage != LBM_STORE_F64 && b->storage != LBM_STORE_DF64_DEV))
    return 1;
  return s;
}

}  // namespace

extern "C" {

int32_t lbm_batch_create(lbm_batch** out, lbm_ctx* const* members, int32_t count) {
  if (!out || !members || count < 1 || count > kBatchMax) return LBM_ERR_INVALID;
  *out = nullptr;
  const lbm_ctx* c0 = members[0];
  if (!c0) return LBM_ERR_INVALID;
  for (int k = 0; k < count; ++k) {
    const lbm_ctx* c = members[k];
    if (!c || c->device != c0->device || c->storage != c0->storage || c->coll != c0->coll) return LBM_ERR_INVALID;
    if (c->coll == LBM_ITERATIVE_INIT) return LBM_ERR_UNSUPPORTED;
    if (c->storage == LBM_STORE_F16_DEV || c->storage == LBM_STORE_F32_DEV_SR || c->storage == LBM_STORE_F64_DD)
      return LBM_ERR_UNSUPPORTED;
  }
  {  // a context may appear once: the batch advances each member's own buffers
    std::vector<lbm_ctx*> sorted(members, members + count);
    std::sort(sorted.begin(), sorted.end());
    if (std::adjacent_find(sorted.begin(), sorted.end()) != sorted.end()) return LBM_ERR_INVALID;
  }
  lbm_batch* b = new lbm_batch();
  b->members.assign(members, members + count);
  for (int k = 0; k < count; ++k) b->time_dependent = b->time_dependent || members[k]->force_kind == LBM_FORCE_SHEAR;
  b->device = c0->device;
  b->storage = c0->storage;
  b->coll = c0->coll;
  DeviceGuard device_guard(b->device);
  const size_t sb = batch_static_size(b->storage);
  std::vector<char> h(sb * count);
  for (int k = 0; k < count; ++k) {
    const lbm_ctx* c = members[k];
    char* slot = h.data() + k * sb;
    if (b->storage == LBM_STORE_F64) fill_static(*reinterpret_cast<BatchStatic<double>*>(slot), c->pd, c);
    else if (b->storage == LBM_STORE_DF64_DEV) fill_static(*reinterpret_cast<BatchStatic<dd>*>(slot), c->px, c);
    else fill_static(*reinterpret_cast<BatchStatic<float>*>(slot), c->pf, c);
  }
  if (cudaDeviceGetAttribute(&b->sm_count, cudaDevAttrMultiProcessorCount, b->device) != cudaSuccess ||
      cudaDeviceGetAttribute(&b->smem_per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, b->device) != cudaSuccess) {
    drop_reported_error();
    b->sm_count = b->smem_per_sm = 0;
  }
  if (!make_stream(&b->own_stream) || !make_event(&b->done) || !make_event(&b->staged) ||
      !dev_malloc(&b->d_static, sb * count) ||
      !dev_malloc((void**)&b->d_dyn, sizeof(BatchDyn) * count) ||
      !host_malloc((void**)&b->h_dyn, sizeof(BatchDyn) * count) ||
      !dev_malloc((void**)&b->d_rdyn, sizeof(ResidentDyn) * count) ||
      !host_malloc((void**)&b->h_rdyn, sizeof(ResidentDyn) * count) ||
      !dev_malloc((void**)&b->d_rout, sizeof(double) * kRedMaxK * count) ||
      !host_malloc((void**)&b->h_rout, sizeof(double) * kRedMaxK * count) ||
      cudaMemcpy(b->d_static, h.data(), sb * count, cudaMemcpyHostToDevice) != cudaSuccess) {
    lbm_batch_destroy(b);
    drop_reported_error();
    return LBM_ERR_NOMEM;
  }
  b->stream = b->own_stream;
  *out = b;
  return LBM_OK;
}

void lbm_batch_destroy(lbm_batch* b) {
  if (!b) return;
  DeviceGuard device_guard(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->shared)
    for (lbm_ctx* c : b->members)
      if (c->stream == b->stream) c->stream = c->own_stream;
  if (b->graph) cudaGraphExecDestroy(b->graph);
  cudaFree(b->d_static);
  cudaFree(b->d_dyn);
  cudaFree(b->d_rdyn);
  if (b->h_rdyn) cudaFreeHost(b->h_rdyn);
  for (cudaEvent_t e : b->res_events) cudaEventDestroy(e);
  if (b->res_fork) cudaEventDestroy(b->res_fork);
  for (cudaStream_t st : b->res_streams) cudaStreamDestroy(st);
  cudaFree(b->d_rargs);
  cudaFree(b->d_rargs_call);
  cudaFree(b->d_ranal);
  if (b->h_ranal) cudaFreeHost(b->h_ranal);
  cudaFree(b->d_rpartial);
  cudaFree(b->d_rout);
  if (b->h_dyn) cudaFreeHost(b->h_dyn);
  if (b->h_rout) cudaFreeHost(b->h_rout);
  if (b->done) cudaEventDestroy(b->done);
  if (b->staged) cudaEventDestroy(b->staged);
  if (b->fork) cudaEventDestroy(b->fork);
  for (cudaEvent_t e : b->group_events) cudaEventDestroy(e);
  for (cudaStream_t st : b->group_streams) cudaStreamDestroy(st);
  if (b->own_stream) cudaStreamDestroy(b->own_stream);
  delete b;
}

const char* lbm_batch_last_error(const lbm_batch* b) { return b ? b->err.c_str() : "null batch"; }
int64_t lbm_batch_last_launch_count(const lbm_batch* b) { return b ? b->last_launches : 0; }

int32_t lbm_batch_set_stream(lbm_batch* b, void* stream) {
  if (!b) return LBM_ERR_INVALID;
  DeviceGuard device_guard(b->device);
  if (cudaStreamSynchronize(b->stream) != cudaSuccess) return bfail(b, LBM_ERR_CUDA, "stream synchronize");
  cudaStream_t next = stream ? static_cast<cudaStream_t>(stream) : b->own_stream;
  if (b->shared)
    for (lbm_ctx* c : b->members)
      if (c->stream == b->stream) c->stream = next;
  b->stream = next;
  if (b->graph) {
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
    b->graph_key.clear();
  }
  return LBM_OK;
}

// Every member issues its own work (uploads, reductions, downloads) on the batch's stream from
// now on, so batch calls need no ordering between streams; the members get their own streams
// back when the batch is destroyed.
int32_t lbm_batch_share_stream(lbm_batch* b) {
  if (!b) return LBM_ERR_INVALID;
  DeviceGuard device_guard(b->device);
  for (lbm_ctx* c : b->members) {
    if (c->stream == b->stream) continue;
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) return bfail(b, LBM_ERR_CUDA, "member synchronize");
    c->stream = b->stream;
  }
  b->shared = true;
  return LBM_OK;
}

int32_t lbm_batch_set_schedule(lbm_batch* b, const lbm_batch_schedule* schedule) {
  if (!b) return LBM_ERR_INVALID;
  if (!schedule) {
    b->schedule = lbm_batch_schedule{};
    return LBM_OK;
  }
  for (int q = 0; q < 7; ++q)
    if (schedule->resident_max_nodes[q] < 0 || schedule->nodes_per_block[q] < 0 || schedule->split[q] < 0)
      return bfail(b, LBM_ERR_INVALID, "schedule: negative limit");
  b->schedule = *schedule;
  return LBM_OK;
}

int32_t lbm_batch_synchronize(lbm_batch* b) {
  if (!b) return LBM_ERR_INVALID;
  DeviceGuard device_guard(b->device);
  return cudaStreamSynchronize(b->stream) == cudaSuccess ? LBM_OK : bfail(b, LBM_ERR_CUDA, "synchronize");
}

// Every member k advances nsteps[k] steps.  All members' steps are issued as ONE CUDA graph of
// kernels, one per global step and velocity set, each covering every member still running.
}  // extern "C"

namespace {

// One call of lbm_batch_step(_timed): t0 / dt (member order) give each member's time index at its
// first step and its time step, or are null for members whose forces do not depend on time.
int batch_step_impl(lbm_batch* b, const int64_t* nsteps, const int64_t* t0, const double* dt) {
  DeviceGuard device_guard(b->device);
  const int count = (int)b->members.size();
  for (int k = 0; k < count; ++k) {
    if (nsteps[k] < 0) return bfail(b, LBM_ERR_INVALID, "negative step count");
    if (!b->members[k]->have_state) return bfail(b, LBM_ERR_STATE, "member without uploaded state");
  }
  // Members that the schedule makes block-resident take all their steps in one launch per
  // (velocity set, cluster size); the others take the graph path with the step counts below.
  std::vector<int> csize(count, 0);
  std::vector<int64_t> gsteps(nsteps, nsteps + count);
  for (int k = 0; k < count; ++k)
    if (nsteps[k] > 0 && (csize[k] = resident_cluster(b, b->members[k])) > 0) gsteps[k] = 0;
  struct ResidentGroup {
    int qid, csize, parts, first, nmem, stride;
  };
  std::vector<ResidentDyn> rdyn;
  std::vector<ResidentGroup> rgroups;
  {
    std::vector<int> res;
    for (int k = 0; k < count; ++k)
      if (csize[k] > 0) res.push_back(k);
    std::stable_sort(res.begin(), res.end(), [&](int a, int c) {
      const int qa = b->members[a]->qid, qc = b->members[c]->qid;
      return qa != qc ? qa < qc : csize[a] < csize[c];
    });
    for (size_t r = 0; r < res.size(); ++r) {
      const int k = res[r];
      const lbm_ctx* c = b->members[k];
      if (rgroups.empty() || rgroups.back().qid != c->qid || rgroups.back().csize != csize[k])
        rgroups.push_back({c->qid, csize[k], resident_parts(b, c), (int)r, 0, 0});
      ResidentGroup& g = rgroups.back();
      ResidentDyn d{};
      d.member = k;
      d.cur0 = c->cur;
      d.phase0 = c->phase == POST_COLLIDE ? 1 : 0;
      d.chunk = (int)((c->n + csize[k] - 1) / csize[k]);
      d.steps = nsteps[k];
      d.t0 = t0 ? (long long)t0[k] : 0;
      d.dt = dt ? dt[k] : 0.0;
      rdyn.push_back(d);
      g.nmem += 1;
      g.stride = std::max(g.stride, d.chunk);
    }
  }
  // graph members grouped by velocity set, each group in descending step order: the running set of
  // a group at global step t is a prefix of it, with block offsets counted within the group
  std::vector<int> order(count);
  for (int k = 0; k < count; ++k) order[k] = k;
  std::stable_sort(order.begin(), order.end(), [&](int a, int c) {
    const int qa = b->members[a]->qid, qc = b->members[c]->qid;
    return qa != qc ? qa < qc : gsteps[a] > gsteps[c];
  });
  std::vector<int64_t> key(count);
  std::vector<long long> end(count, 0);  // end of each member's block range in its group
  std::vector<int> group_begin;          // first rank of each velocity-set group
  std::vector<BatchDyn> dyn(count);
  for (int r = 0; r < count; ++r) {
    const lbm_ctx* c = b->members[order[r]];
    key[r] = gsteps[order[r]];
    const bool first = r == 0 || b->members[order[r - 1]]->qid != c->qid;
    if (first) group_begin.push_back(r);
    BatchDyn& d = dyn[r];
    d.block_start = first ? 0 : end[r - 1];
    d.steps = key[r];
    d.member = order[r];
    d.cur0 = c->cur;
    d.phase0 = c->phase == POST_COLLIDE ? 1 : 0;
    d.pad = 0;
    d.t0 = t0 ? (long long)t0[order[r]] : 0;
    d.dt = dt ? dt[order[r]] : 0.0;
    end[r] = d.block_start + (c->n + batch_block_nodes(b->storage) - 1) / batch_block_nodes(b->storage);
  }
  group_begin.push_back(count);
  int64_t tmax = 0;
  for (int r = 0; r < count; ++r) tmax = std::max(tmax, key[r]);
  b->last_launches = 0;
  if (tmax == 0 && rgroups.empty()) return LBM_OK;
  int rc = batch_wait_members(b);
  if (rc) return rc;
  rc = batch_upload_dyn(b, dyn, rdyn);
  if (rc) return rc;
  if (!rgroups.empty()) {  // resident launches on their own streams, concurrent with the graph
    if (!b->res_fork && !make_event(&b->res_fork)) return bfail(b, LBM_ERR_CUDA, "event");
    while (b->res_streams.size() < rgroups.size()) {
      cudaStream_t st = nullptr;
      if (!make_stream(&st)) return bfail(b, LBM_ERR_CUDA, "resident stream");
      b->res_streams.push_back(st);
    }
    while (b->res_events.size() < rgroups.size()) {
      cudaEvent_t ev = nullptr;
      if (!make_event(&ev)) return bfail(b, LBM_ERR_CUDA, "resident event");
      b->res_events.push_back(ev);
    }
    if (cudaEventRecord(b->res_fork, b->stream) != cudaSuccess) return bfail(b, LBM_ERR_CUDA, "resident fork");
    // When every CTA of the call can have an SM of its own, each asks for more than half an SM's
    // shared memory, so that no two share an SM's FP64 units: a small member's step is bound by
    // the latency of its warps' collision chains, which a second CTA on the SM would lengthen
    // (a launch whose clusters would not all fit at once that way keeps its own size).
    long long ctas = 0;
    for (const ResidentGroup& g : rgroups) ctas += (long long)g.nmem * g.csize;
    const size_t smem_min = (b->sm_count > 0 && ctas <= b->sm_count) ? (size_t)b->smem_per_sm / 2 + 1024 : 0;
    for (size_t gi = 0; gi < rgroups.size(); ++gi) {
      const ResidentGroup& g = rgroups[gi];
      cudaStream_t st = b->res_streams[gi];
      // node groups of 32 (one node per lane), each on `parts` warps, at most kResidentThreads threads
      const int groups = std::max(1, std::min((g.stride + 31) / 32, kResidentThreads / (32 * g.parts)));
      const int threads = groups * 32 * g.parts;
      cudaError_t e = cudaStreamWaitEvent(st, b->res_fork, 0);
      if (e == cudaSuccess)
        e = resident_launch(b->storage, b->coll, g.qid, b->d_static, b->d_rdyn + g.first, g.nmem, g.csize, g.stride,
                            threads, g.parts, smem_min, st);
      if (e == cudaSuccess) e = cudaEventRecord(b->res_events[gi], st);
      if (e != cudaSuccess) {
        char what[200];
        std::snprintf(what, sizeof what, "resident launch (velocity set %d, %d members, clusters of %d CTAs x %d threads, "
                      "%d nodes per plane, %d warps per node): ", g.qid, g.nmem, g.csize, threads, g.stride, g.parts);
        return bfail(b, LBM_ERR_CUDA, std::string(what) + cudaGetErrorString(e));
      }
    }
  }
  b->res_launches = (int64_t)rgroups.size();
  if (tmax > 0) {
  if (!b->graph || b->graph_key != key || b->graph_order != order) {
    if (b->graph) {
      cudaGraphExecDestroy(b->graph);
      b->graph = nullptr;
    }
    const int ngroups = (int)group_begin.size() - 1;
    // the velocity-set groups advance independently: with more than one, each group's chain of
    // steps is captured on its own stream, forked from and joined to the batch stream, so that
    // the graph runs the chains concurrently
    if (ngroups > 1) {  // streams and events are kept when a later one fails, so each is counted on its own
      if (!b->fork && !make_event(&b->fork)) return bfail(b, LBM_ERR_CUDA, "event");
      while ((int)b->group_streams.size() < ngroups) {
        cudaStream_t st = nullptr;
        if (!make_stream(&st)) return bfail(b, LBM_ERR_CUDA, "group stream");
        b->group_streams.push_back(st);
      }
      while ((int)b->group_events.size() < ngroups) {
        cudaEvent_t ev = nullptr;
        if (!make_event(&ev)) return bfail(b, LBM_ERR_CUDA, "group event");
        b->group_events.push_back(ev);
      }
    }
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
      return bfail(b, LBM_ERR_CUDA, "begin capture");
    cudaError_t e = cudaSuccess;
    if (ngroups > 1) {
      e = cudaEventRecord(b->fork, b->stream);
      for (int gi = 0; gi < ngroups && e == cudaSuccess; ++gi) e = cudaStreamWaitEvent(b->group_streams[gi], b->fork, 0);
    }
    int64_t launches = 0;
    for (int gi = 0; gi < ngroups && e == cudaSuccess; ++gi) {
      const int g0 = group_begin[gi];
      cudaStream_t st = ngroups > 1 ? b->group_streams[gi] : b->stream;
      int nactive = group_begin[gi + 1] - g0;
      for (int64_t t = 0; t < key[g0] && e == cudaSuccess; ++t) {  // key[g0]: the group's most steps
        while (nactive > 0 && key[g0 + nactive - 1] <= t) --nactive;
        e = batch_launch(b->storage, b->coll, b->members[order[g0]]->qid, b->d_static, b->d_dyn + g0, nactive,
                         end[g0 + nactive - 1], t, st);
        ++launches;
      }
      if (ngroups > 1 && e == cudaSuccess) {
        e = cudaEventRecord(b->group_events[gi], st);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(b->stream, b->group_events[gi], 0);
      }
    }
    cudaError_t e2 = cudaStreamEndCapture(b->stream, &g);
    if (e != cudaSuccess || e2 != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      return bfail(b, LBM_ERR_CUDA, std::string("batch capture: ") + cudaGetErrorString(e != cudaSuccess ? e : e2));
    }
    e = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
      b->graph = nullptr;
      return bfail(b, LBM_ERR_CUDA, std::string("batch graph: ") + cudaGetErrorString(e));
    }
    b->graph_key = key;
    b->graph_order = order;
    b->graph_launches = launches;
  }
  if (cudaGraphLaunch(b->graph, b->stream) != cudaSuccess) return bfail(b, LBM_ERR_CUDA, "graph launch");
  b->last_launches = b->graph_launches;
  }  // tmax > 0
  for (size_t gi = 0; gi < rgroups.size(); ++gi)  // join the resident launches
    if (cudaStreamWaitEvent(b->stream, b->res_events[gi], 0) != cudaSuccess)
      return bfail(b, LBM_ERR_CUDA, "resident join");
  b->last_launches += b->res_launches;
  // members continue after the batch: advance their parity / phase and order their streams
  for (int k = 0; k < count; ++k) {
    lbm_ctx* c = b->members[k];
    if (nsteps[k] > 0) {
      c->cur = (int)((c->cur + nsteps[k]) & 1);
      c->phase = POST_COLLIDE;
    }
  }
  return batch_release_members(b);
}

}  // namespace

extern "C" {

int32_t lbm_batch_step(lbm_batch* b, const int64_t* nsteps) {
  if (!b || !nsteps) return LBM_ERR_INVALID;
  if (b->time_dependent)
    return bfail(b, LBM_ERR_INVALID, "a member's force depends on time: step with lbm_batch_step_timed");
  return batch_step_impl(b, nsteps, nullptr, nullptr);
}

int32_t lbm_batch_step_timed(lbm_batch* b, const int64_t* nsteps, const int64_t* t0, const double* dt) {
  if (!b || !nsteps || !t0 || !dt) return LBM_ERR_INVALID;
  return batch_step_impl(b, nsteps, t0, dt);
}

}  // extern "C"

namespace {

// Per-member reduction arguments (weights, 1/c_s², previous-velocity planes), built once.
int batch_ensure_rargs(lbm_batch* b) {
  if (b->d_rargs) return LBM_OK;
  const int count = (int)b->members.size();
  b->h_rargs.resize(count);
  for (int k = 0; k < count; ++k) {
    lbm_ctx* c = b->members[k];
    if (!c->d_uold) {
      if (ensure(c, &c->d_uold, (size_t)c->n * 2 * sizeof(double))) return bfail(b, LBM_ERR_NOMEM, c->err);
      if (cudaMemsetAsync(c->d_uold, 0, (size_t)c->n * 2 * sizeof(double), b->stream) != cudaSuccess)
        return bfail(b, LBM_ERR_CUDA, "previous-velocity planes");
    }
    b->h_rargs[k] = c->red;
    b->h_rargs[k].u_old = c->d_uold;
  }
  if (!dev_malloc((void**)&b->d_rargs, sizeof(ReduceArgs) * count))
    return bfail(b, LBM_ERR_NOMEM, "reduction arguments");
  if (cudaMemcpy(b->d_rargs, b->h_rargs.data(), sizeof(ReduceArgs) * count, cudaMemcpyHostToDevice) != cudaSuccess)
    return bfail(b, LBM_ERR_CUDA, "reduction arguments");
  return LBM_OK;
}

// The selected members' K sums of one reduction kind, with the arguments array `args`.
int batch_reduce_run(lbm_batch* b, int K, const std::vector<int>& selected, const ReduceArgs* args, double* out) {
  const int count = (int)b->members.size();
  std::vector<int> order = selected;
  std::stable_sort(order.begin(), order.end(),
                   [&](int a, int c) { return b->members[a]->qid < b->members[c]->qid; });
  const int nsel = (int)order.size();
  std::fill(out, out + (size_t)count * kRedMaxK, 0.0);
  if (nsel == 0) return LBM_OK;
  std::vector<BatchDyn> dyn(nsel);
  std::vector<int> group_begin;
  std::vector<long long> group_base;  // first partial block of each group
  long long total = 0, gstart = 0;
  for (int r = 0; r < nsel; ++r) {
    const lbm_ctx* c = b->members[order[r]];
    const bool first = r == 0 || b->members[order[r - 1]]->qid != c->qid;
    if (first) {
      group_begin.push_back(r);
      group_base.push_back(total);
      gstart = 0;
    }
    const long long nb = c->red_blocks;  // lbm_reduce's partition, so the sums are bitwise the same
    BatchDyn& d = dyn[r];
    d.block_start = gstart;
    d.steps = nb;
    d.member = order[r];
    d.cur0 = c->cur;
    d.phase0 = c->phase == POST_COLLIDE ? 1 : 0;
    d.pad = 0;
    gstart += nb;
    total += nb;
  }
  group_begin.push_back(nsel);
  if (total > b->rpartial_blocks) {
    cudaFree(b->d_rpartial);
    b->d_rpartial = nullptr;
    if (!dev_malloc((void**)&b->d_rpartial, sizeof(double) * kRedMaxK * total)) {
      b->rpartial_blocks = 0;
      return bfail(b, LBM_ERR_NOMEM, "reduction partials");
    }
    b->rpartial_blocks = total;
  }
  int rc = batch_upload_dyn(b, dyn, {});
  if (rc) return rc;
  for (size_t gi = 0; gi + 1 < group_begin.size(); ++gi) {
    const int g0 = group_begin[gi], n = group_begin[gi + 1] - g0;
    const long long blocks = dyn[group_begin[gi + 1] - 1].block_start + dyn[group_begin[gi + 1] - 1].steps;
    cudaError_t e = batch_reduce_launch(b->storage, b->members[order[g0]]->qid, K, b->d_static, args, b->d_dyn + g0, n,
                                        blocks, b->d_rpartial, group_base[gi], b->d_rout, b->stream);
    if (e != cudaSuccess) return bfail(b, LBM_ERR_CUDA, std::string("batched reduction: ") + cudaGetErrorString(e));
  }
  if (cudaMemcpyAsync(b->h_rout, b->d_rout, sizeof(double) * kRedMaxK * count, cudaMemcpyDeviceToHost, b->stream) !=
          cudaSuccess ||
      cudaStreamSynchronize(b->stream) != cudaSuccess)
    return bfail(b, LBM_ERR_CUDA, "batched reduction result");
  for (int k : order)
    for (int j = 0; j < K; ++j) out[(size_t)k * kRedMaxK + j] = b->h_rout[(size_t)k * kRedMaxK + j];
  return LBM_OK;
}

}  // namespace

extern "C" {

// The reductions lbm_reduce computes without analytic fields (MEAN_VELOCITY,
// VELOCITY_CONVERGENCE, CONSERVED) for the selected members at once: out[k * 16 + j] is what
// lbm_reduce(member k, kind) would return in out[j].  One launch per velocity set plus one
// fixed-order finish; VELOCITY_CONVERGENCE updates each member's previous-velocity planes as
// lbm_reduce does.  CONSERVED reports the non-finite population count in out[k * 16 + 3].
int32_t lbm_batch_reduce(lbm_batch* b, int32_t kind, const uint8_t* select, double* out) {
  if (!b || !out) return LBM_ERR_INVALID;
  if (kind != LBM_REDUCE_MEAN_VELOCITY && kind != LBM_REDUCE_VELOCITY_CONVERGENCE && kind != LBM_REDUCE_CONSERVED)
    return bfail(b, LBM_ERR_UNSUPPORTED, "batched reductions: MEAN_VELOCITY, VELOCITY_CONVERGENCE, CONSERVED");
  DeviceGuard device_guard(b->device);
  const int count = (int)b->members.size();
  std::vector<int> selected;
  for (int k = 0; k < count; ++k)
    if (!select || select[k]) {
      if (!b->members[k]->have_state) return bfail(b, LBM_ERR_STATE, "member without uploaded state");
      selected.push_back(k);
    }
  int rc = batch_wait_members(b);
  if (rc) return rc;
  rc = batch_ensure_rargs(b);
  if (rc) return rc;
  rc = batch_reduce_run(b, red_kind_k(kind), selected, b->d_rargs, out);
  if (rc) return rc;
  return batch_release_members(b);
}

// The error-norm reductions with analytic fields (TRACK_ERRORS, COMPARE) for the selected
// members at once; analytic[k] holds member k's host planes and scalars as lbm_reduce takes them.
int32_t lbm_batch_reduce_fields(lbm_batch* b, int32_t kind, const uint8_t* select, const lbm_analytic* analytic,
                                double* out) {
  if (!b || !out || !analytic) return LBM_ERR_INVALID;
  if (kind != LBM_REDUCE_TRACK_ERRORS && kind != LBM_REDUCE_COMPARE)
    return bfail(b, LBM_ERR_UNSUPPORTED, "batched field reductions: TRACK_ERRORS, COMPARE");
  DeviceGuard device_guard(b->device);
  const int count = (int)b->members.size();
  const int need = kind == LBM_REDUCE_TRACK_ERRORS ? 8 : 4;
  std::vector<int> selected;
  size_t total = 0;
  for (int k = 0; k < count; ++k) {
    if (select && !select[k]) continue;
    const lbm_analytic& an = analytic[k];
    const double* src[8] = {an.rho, an.ux, an.uy, an.p, an.sxx, an.syx, an.sxy, an.syy};
    if (!b->members[k]->have_state) return bfail(b, LBM_ERR_STATE, "member without uploaded state");
    if (an.on_device) return bfail(b, LBM_ERR_UNSUPPORTED, "batched field reductions take host planes");
    for (int j = 0; j < need; ++j)
      if (!src[j]) return bfail(b, LBM_ERR_INVALID, "missing analytic field");
    selected.push_back(k);
    total += (size_t)need * b->members[k]->n;
  }
  int rc = batch_wait_members(b);
  if (rc) return rc;
  rc = batch_ensure_rargs(b);
  if (rc) return rc;
  if (total > b->ranal_cap) {
    cudaFree(b->d_ranal);
    if (b->h_ranal) cudaFreeHost(b->h_ranal);
    b->d_ranal = nullptr;
    b->h_ranal = nullptr;
    b->ranal_cap = 0;
    if (!dev_malloc((void**)&b->d_ranal, total * sizeof(double)) ||
        !host_malloc((void**)&b->h_ranal, total * sizeof(double)))
      return bfail(b, LBM_ERR_NOMEM, "analytic staging");
    b->ranal_cap = total;
  }
  if (!b->d_rargs_call && !dev_malloc((void**)&b->d_rargs_call, sizeof(ReduceArgs) * count))
    return bfail(b, LBM_ERR_NOMEM, "reduction arguments");
  // pack the planes (the pinned staging is free: the previous call ended with a synchronize)
  std::vector<ReduceArgs> args = b->h_rargs;
  size_t off = 0;
  for (int k : selected) {
    const lbm_analytic& an = analytic[k];
    const double* src[8] = {an.rho, an.ux, an.uy, an.p, an.sxx, an.syx, an.sxy, an.syy};
    const size_t n = (size_t)b->members[k]->n;
    const double* dp[8] = {};
    for (int j = 0; j < need; ++j) {
      std::memcpy(b->h_ranal + off, src[j], n * sizeof(double));
      dp[j] = b->d_ranal + off;
      off += n;
    }
    ReduceArgs& r = args[k];
    r.rho_a = dp[0];
    r.ux_a = dp[1];
    r.uy_a = dp[2];
    r.p_a = dp[3];
    r.sxx_a = dp[4];
    r.syx_a = dp[5];
    r.sxy_a = dp[6];
    r.syy_a = dp[7];
    r.tau = an.tau;
    r.u_max = an.u_max;
    r.area = an.area;
  }
  if ((total && cudaMemcpyAsync(b->d_ranal, b->h_ranal, total * sizeof(double), cudaMemcpyHostToDevice, b->stream) !=
                    cudaSuccess) ||
      cudaMemcpyAsync(b->d_rargs_call, args.data(), sizeof(ReduceArgs) * count, cudaMemcpyHostToDevice, b->stream) !=
          cudaSuccess)
    return bfail(b, LBM_ERR_CUDA, "analytic upload");
  rc = batch_reduce_run(b, red_kind_k(kind), selected, b->d_rargs_call, out);
  // the pageable argument copy above completes before its call returns; the pinned planes
  // were synchronised by the result read
  if (rc) return rc;
  return batch_release_members(b);
}

}  // extern "C"

// ---- adjoint -------------------------------------------------------------------------------

// One action of the adjoint's plan.  A location names a state buffer: kLocA0 (A_0), kLocWork + w
// (two work buffers) or a checkpoint slot (>= 0).
struct AdjAction {
  enum Kind { FWD, LOSS, ADJ } kind;
  int src, dst;  // FWD: src -> dst (one step); LOSS: src holds B_{T-1}; ADJ: src holds the state entering t
  int64_t t;     // FWD: the step's time index (0: the collision-only first step); ADJ: the reversed step
};
constexpr int kLocA0 = -1, kLocWork = -3;  // work buffers: kLocWork + 0, kLocWork + 1 (= -3, -2)

struct lbm_adjoint {
  lbm_ctx* ctx = nullptr;
  int64_t T = 0, nslots = 0;
  size_t bytes = 0;
  int nblocks = 0;
  void* a0 = nullptr;
  void* work[2] = {nullptr, nullptr};
  std::vector<void*> slot;      // checkpoints of the binomial schedule
  std::vector<AdjAction> plan;  // the forward, loss and reverse steps, in order
  int64_t forward_steps = 0;    // forward steps of the plan (T without checkpointing)
  void* lam[2] = {nullptr, nullptr};
  double* d_u0 = nullptr;
  double* d_ut = nullptr;
  double* d_grad = nullptr;
  double* d_slots = nullptr;   // loss: nblocks x 1, then parameters: nblocks x 5
  double* d_out = nullptr;     // loss, dω_s, dω_a, dτ_a(force), dF_x, dF_y
  double* h_out = nullptr;
  cudaGraphExec_t graph = nullptr;
  cudaStream_t graph_stream = nullptr;
  std::string err;
};

namespace {

// β(s, r) = C(s + r, s): the most steps that s checkpoints reverse with every step recomputed at
// most r times (Griewank, "Achieving logarithmic growth of temporal and spatial complexity in
// reverse automatic differentiation", 1992), saturated at 2^62.
int64_t binomial_beta(int64_t s, int64_t r) {
  double b = 1.0;
  for (int64_t j = 1; j <= s; ++j) {
    b = b * (double)(r + j) / (double)j;
    if (b > 4.6e18) return int64_t(1) << 62;
  }
  return (int64_t)(b + 0.5);
}

// The plan of the binomial (revolve-type) checkpointing schedule.  reverse(start, t0, t1, s):
// the state entering step t0 is at `start`, λ_{t1} is known (or, on the rightmost path, still to
// be formed by the loss), and s slots are free.  With r the least repetition count such that
// β(s, r) >= n = t1 - t0, the state entering t0 + m is kept in a slot, where m takes the
// largest value that leaves the right part n - m steps with s - 1 slots and r repetitions
// (n - m <= β(s - 1, r)) and the left part m steps with s slots and r - 1 repetitions
// (m <= β(s, r - 1)); since β(s, r) = β(s - 1, r) + β(s, r - 1), such m exists.  The right part is
// reversed first, then the left one from `start`.  Without free slots, each state is recomputed
// from `start`.
struct AdjPlanner {
  std::vector<AdjAction>& out;
  int64_t T;
  int64_t fwd = 0;
  std::vector<bool> used;

  // forward from the state entering t_from (at `from`) to the state entering t_to, the last step
  // into `dst` (or a work buffer when dst is kLocWork), returning the location
  int advance(int from, int64_t t_from, int64_t t_to, int dst) {
    int cur = from;
    for (int64_t t = t_from; t < t_to; ++t) {
      int next;
      if (t + 1 == t_to && dst != kLocWork) next = dst;
      else next = (cur == kLocWork) ? kLocWork + 1 : kLocWork;  // the work buffer not read now
      out.push_back({AdjAction::FWD, cur, next, t});
      ++fwd;
      cur = next;
    }
    return cur;
  }
  int take_slot() {
    for (size_t j = 0; j < used.size(); ++j)
      if (!used[j]) {
        used[j] = true;
        return (int)j;
      }
    return -100;  // not reached: the recursion never holds more slots than it was given
  }
  void adj(int64_t t, int src) { out.push_back({AdjAction::ADJ, src, 0, t}); }
  void loss_from(int start, int64_t t_start) {  // B_{T-1} from the state entering t_start
    const int loc = advance(start, t_start, T, kLocWork);
    out.push_back({AdjAction::LOSS, loc, 0, T});
  }
  void reverse(int start, int64_t t0, int64_t t1, int64_t s, bool need_loss) {
    const int64_t n = t1 - t0;
    if (n == 1 || s == 0) {
      if (need_loss) loss_from(start, t0);
      for (int64_t t = t1 - 1; t >= t0; --t) adj(t, t == t0 ? start : advance(start, t0, t, kLocWork));
      return;
    }
    int64_t r = 1;
    while (binomial_beta(s, r) < n) ++r;
    int64_t m = std::min<int64_t>(binomial_beta(s, r - 1), n - 1);
    m = std::max<int64_t>(m, std::max<int64_t>(1, n - binomial_beta(s - 1, r)));
    const int sl = take_slot();
    advance(start, t0, t0 + m, sl);
    reverse(sl, t0 + m, t1, s - 1, need_loss);
    used[sl] = false;
    reverse(start, t0, t0 + m, s, false);
  }
};

int afail(lbm_adjoint* a, int status, const std::string& msg) {
  if (a) a->err = msg;
  drop_if_cuda(status);
  return status;
}

const void* ctx_params(lbm_ctx* c) {
  return c->storage == LBM_STORE_F64 ? static_cast<const void*>(&c->pd) : static_cast<const void*>(&c->pf);
}

// The plan's forward steps, loss and reverse steps, then ∂L/∂u0 and the sensitivity sums.
cudaError_t adjoint_sequence(lbm_adjoint* a) {
  lbm_ctx* c = a->ctx;
  cudaStream_t s = c->stream;
  const int nb = a->nblocks;
  AdjArgs args{};
  args.Fx = c->force_kind == LBM_FORCE_CONSTANT ? c->pd.F[0] : 0.0;
  args.Fy = c->force_kind == LBM_FORCE_CONSTANT ? c->pd.F[1] : 0.0;
  args.shift = c->pd.shift;
  const void* prm = ctx_params(c);
  double* loss_slots = a->d_slots;
  double* par_slots = a->d_slots + nb;
  auto loc = [&](int l) -> void* {
    if (l == kLocA0) return a->a0;
    if (l == kLocWork || l == kLocWork + 1) return a->work[l - kLocWork];
    return a->slot[(size_t)l];
  };
  cudaError_t e = cudaMemsetAsync(a->d_slots, 0, (size_t)nb * (1 + kAdjParams) * sizeof(double), s);
  if (e != cudaSuccess) return e;
  // A_0
  e = adj_launch(0, c->qid, c->storage, c->coll, prm, args, nullptr, 0, nullptr, a->a0, nullptr, nb, a->d_u0, nullptr,
                 nullptr, s);
  if (e != cudaSuccess) return e;
  for (const AdjAction& x : a->plan) {
    if (x.kind == AdjAction::FWD) {  // B_t from the state entering step t (A_0 for t = 0: collision only)
      OpArgs o = base_args(c, x.t == 0 ? OP_COLLIDE : OP_FUSED);
      o.src = loc(x.src);
      o.dst = loc(x.dst);
      o.stream = s;
      e = kRun[c->qid](o);
    } else if (x.kind == AdjAction::LOSS) {  // loss and λ_T from A_T = S(B_{T-1})
      e = adj_launch(1, c->qid, c->storage, c->coll, prm, args, loc(x.src), 1, nullptr, a->lam[a->T & 1], loss_slots,
                     nb, nullptr, a->d_ut, nullptr, s);
    } else {  // λ_t from λ_{t+1} and A_t (pulled from B_{t-1}, or A_0 read as it is)
      e = adj_launch(2, c->qid, c->storage, c->coll, prm, args, loc(x.src), x.t == 0 ? 0 : 1, a->lam[(x.t + 1) & 1],
                     a->lam[x.t & 1], par_slots, nb, nullptr, nullptr, nullptr, s);
    }
    if (e != cudaSuccess) return e;
  }
  e = adj_launch(3, c->qid, c->storage, c->coll, prm, args, nullptr, 0, a->lam[0], nullptr, nullptr, nb, a->d_u0,
                 nullptr, a->d_grad, s);
  if (e != cudaSuccess) return e;
  e = adj_finish(loss_slots, nb, 1, a->d_out, s);
  if (e != cudaSuccess) return e;
  return adj_finish(par_slots, nb, kAdjParams, a->d_out + 1, s);
}

}  // namespace

extern "C" {

int32_t lbm_adjoint_create(lbm_adjoint** out, lbm_ctx* c, int64_t nsteps, int64_t slots) {
  if (!out || !c || nsteps < 1 || slots < 0) return LBM_ERR_INVALID;
  *out = nullptr;
  if (c->qid != LBM_D2Q9 && c->qid != LBM_D2Q13) return fail(c, LBM_ERR_UNSUPPORTED, "adjoint: D2Q9 / D2Q13 only");
  if (c->coll != LBM_SRT && c->coll != LBM_TRT && c->coll != LBM_MRT)
    return fail(c, LBM_ERR_UNSUPPORTED, "adjoint: SRT / TRT / MRT only");
  if (c->storage != LBM_STORE_F64 && c->storage != LBM_STORE_F32_DEV)
    return fail(c, LBM_ERR_UNSUPPORTED, "adjoint: FP64 or FP32-deviation storage only");
  if (c->force_kind != LBM_FORCE_NONE && c->force_kind != LBM_FORCE_CONSTANT)
    return fail(c, LBM_ERR_UNSUPPORTED, "adjoint: uniform force only");
  DeviceGuard device_guard(c->device);
  lbm_adjoint* a = new lbm_adjoint();
  a->ctx = c;
  a->T = nsteps;
  // default: the fewest slots with which no step is recomputed more than twice
  int64_t sl = slots;
  if (sl == 0) {
    sl = 1;
    while (binomial_beta(sl, 2) < nsteps) ++sl;
  }
  a->nslots = std::min<int64_t>(sl, std::max<int64_t>(nsteps - 1, 0));
  {
    AdjPlanner pl{a->plan, a->T};
    pl.used.assign((size_t)a->nslots, false);
    pl.reverse(kLocA0, 0, a->T, a->nslots, true);
    a->forward_steps = pl.fwd;
  }
  a->bytes = (size_t)c->n * c->Q * c->elem;
  a->nblocks = (int)std::min<int64_t>((c->n + kAdjThreads - 1) / kAdjThreads, kSumBlocks);
  bool ok = dev_malloc(&a->a0, a->bytes) && dev_malloc(&a->work[0], a->bytes) &&
            dev_malloc(&a->work[1], a->bytes) && dev_malloc(&a->lam[0], a->bytes) &&
            dev_malloc(&a->lam[1], a->bytes) &&
            dev_malloc(&a->d_u0, (size_t)c->n * 2 * sizeof(double)) &&
            dev_malloc(&a->d_ut, (size_t)c->n * 2 * sizeof(double)) &&
            dev_malloc(&a->d_grad, (size_t)c->n * 2 * sizeof(double)) &&
            dev_malloc(&a->d_slots, (size_t)a->nblocks * (1 + kAdjParams) * sizeof(double)) &&
            dev_malloc(&a->d_out, 8 * sizeof(double)) &&
            host_malloc(&a->h_out, 8 * sizeof(double));
  a->slot.assign((size_t)a->nslots, nullptr);
  for (int64_t j = 0; ok && j < a->nslots; ++j) ok = dev_malloc(&a->slot[(size_t)j], a->bytes);
  if (!ok) {
    lbm_adjoint_destroy(a);
    return fail(c, LBM_ERR_NOMEM, "adjoint: device memory for checkpoints");
  }
  *out = a;
  return LBM_OK;
}

int32_t lbm_adjoint_info(const lbm_adjoint* a, int64_t* slots, int64_t* forward_steps, int64_t* device_bytes) {
  if (!a) return LBM_ERR_INVALID;
  if (slots) *slots = a->nslots;
  if (forward_steps) *forward_steps = a->forward_steps;
  if (device_bytes)  // states (A_0, two work buffers, the slots, two adjoint states) and the planes
    *device_bytes = (int64_t)(a->bytes * (size_t)(5 + a->nslots) + (size_t)a->ctx->n * 6 * sizeof(double) +
                              (size_t)a->nblocks * (1 + kAdjParams) * sizeof(double) + 8 * sizeof(double));
  return LBM_OK;
}

void lbm_adjoint_destroy(lbm_adjoint* a) {
  if (!a) return;
  DeviceGuard device_guard(a->ctx->device);
  cudaStreamSynchronize(a->ctx->stream);
  if (a->graph) cudaGraphExecDestroy(a->graph);
  void* bufs[] = {a->a0, a->work[0], a->work[1], a->lam[0], a->lam[1], a->d_u0, a->d_ut, a->d_grad, a->d_slots, a->d_out};
  for (void* b : bufs) cudaFree(b);
  for (void* b : a->slot) cudaFree(b);
  if (a->h_out) cudaFreeHost(a->h_out);
  delete a;
}

const char* lbm_adjoint_last_error(const lbm_adjoint* a) { return a ? a->err.c_str() : "null adjoint"; }

int32_t lbm_adjoint_run(lbm_adjoint* a, const double* u0, const double* u_target, double* result,
                        double* grad_u0) {
  if (!a || !u0 || !u_target || !result) return LBM_ERR_INVALID;
  lbm_ctx* c = a->ctx;
  DeviceGuard device_guard(c->device);
  cudaStream_t s = c->stream;
  const size_t vb = (size_t)c->n * 2 * sizeof(double);
  if (cudaMemcpyAsync(a->d_u0, u0, vb, cudaMemcpyDefault, s) != cudaSuccess ||
      cudaMemcpyAsync(a->d_ut, u_target, vb, cudaMemcpyDefault, s) != cudaSuccess)
    return afail(a, LBM_ERR_CUDA, "adjoint: input copies");
  if (!a->graph || a->graph_stream != s) {
    if (a->graph) {
      cudaGraphExecDestroy(a->graph);
      a->graph = nullptr;
    }
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
      return afail(a, LBM_ERR_CUDA, "adjoint: begin capture");
    cudaError_t e = adjoint_sequence(a);
    cudaError_t e2 = cudaStreamEndCapture(s, &g);
    if (e != cudaSuccess || e2 != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      return afail(a, LBM_ERR_CUDA, std::string("adjoint capture: ") + cudaGetErrorString(e != cudaSuccess ? e : e2));
    }
    e = cudaGraphInstantiate(&a->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
      a->graph = nullptr;
      return afail(a, LBM_ERR_CUDA, std::string("adjoint graph: ") + cudaGetErrorString(e));
    }
    a->graph_stream = s;
  }
  if (cudaGraphLaunch(a->graph, s) != cudaSuccess) return afail(a, LBM_ERR_CUDA, "adjoint: graph launch");
  c->last_launches = (int64_t)a->plan.size() + 5;
  if (cudaMemcpyAsync(a->h_out, a->d_out, 6 * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return afail(a, LBM_ERR_CUDA, "adjoint: result copy");
  if (grad_u0 && cudaMemcpyAsync(grad_u0, a->d_grad, vb, cudaMemcpyDefault, s) != cudaSuccess)
    return afail(a, LBM_ERR_CUDA, "adjoint: gradient copy");
  if (cudaStreamSynchronize(s) != cudaSuccess) return afail(a, LBM_ERR_CUDA, "adjoint: synchronize");
  // result: loss, dL/dτ_s, dL/dτ_a, dL/dF_x, dL/dF_y (partial derivatives; SRT: dL/dτ in [1] and [2] summed;
  // MRT: dL/dτ_2 in [1], the second-order relaxation time, which also scales the force shift)
  const double* h = a->h_out;
  const double ts = c->coll == LBM_TRT ? 1.0 / c->pd.inv_ts
                  : c->coll == LBM_MRT ? 1.0 / c->pd.mrt_b[1] : 1.0 / c->pd.om_b;
  const double ta = c->coll == LBM_TRT ? 1.0 / c->pd.inv_ta : ts;
  result[0] = h[0];
  if (c->coll == LBM_TRT) {
    result[1] = h[1] * (-1.0 / (ts * ts));
    result[2] = h[2] * (-1.0 / (ta * ta)) + h[3];
  } else {
    result[1] = (h[1] + h[2]) * (-1.0 / (ts * ts)) + h[3];
    result[2] = 0.0;
  }
  result[3] = h[4];
  result[4] = h[5];
  return LBM_OK;
}

}  // extern "C"
