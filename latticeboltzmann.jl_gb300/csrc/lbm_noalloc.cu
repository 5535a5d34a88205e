// lbm_noalloc.cu -- the processing-method reductions for callers that cannot allocate device
// memory.
//
// lbm_reduce needs a context, and creating one allocates (population buffers, the partial-sum
// buffer of the reduction).  Some callers cannot do that: code running inside a CUDA-graph
// capture or another library's stream callback, hosts whose device memory is owned by a pool
// they may not grow (a Julia CuArray pool, an embedding that forbids cudaMalloc while it holds
// the device), or a failure path where an allocation would itself fail.  They hold the
// populations already and only want the sums.  lbm_reduce_noalloc takes the populations, the
// analytic fields and the output as device pointers the caller owns and keeps its one piece of
// scratch -- one partial sum per block -- in the file-scope device array below.
//
// The array is a static device variable: every GPU that loads this library holds its 77,824
// bytes until the process exits.  Host code cannot use the name of the array as a device
// address (it names a host-side stand-in), so each device's address is looked up once with
// cudaGetSymbolAddress, with that device current, the first time the entry point runs on it.
// The cached address belongs to the device's context: it does not survive cudaDeviceReset (or
// any other teardown of the primary context), after which this entry point must not be called
// again in the process.
//
// Reductions run in the same kernels, grid size and fixed block order as lbm_reduce, so for
// the same populations the two entry points return the same sums.
#include <algorithm>
#include <mutex>

#include "lbm_ops.cuh"

namespace {

constexpr int kNoAllocBlocks = lbm::kSumBlocks;  // the partition of lbm_reduce: the same bits
constexpr int kNoAllocSlots = kNoAllocBlocks * lbm::kRedMaxK;

static __device__ __align__(256) double g_noalloc_partial[kNoAllocSlots];

constexpr int kMaxDevices = 64;
std::mutex g_addr_mutex;
double* g_addr[kMaxDevices] = {};

// Device address of g_noalloc_partial on the current device (looked up once per device).
cudaError_t scratch_address(double** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_addr_mutex);
  if (!g_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_partial);
    if (e != cudaSuccess) return e;
    g_addr[dev] = static_cast<double*>(p);
  }
  *out = g_addr[dev];
  return cudaSuccess;
}

// The kernel runs on the current device, so every array it reads or writes must be memory of that
// device: a pointer into another GPU's memory, or into host memory the runtime does not know, is
// refused before the launch (cudaPointerGetAttributes allocates nothing).
bool on_device(const void* ptr, int dev) {
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, ptr) != cudaSuccess) {
    (void)cudaGetLastError();
    return false;
  }
  if (at.type == cudaMemoryTypeDevice) return at.device == dev;
  return at.type == cudaMemoryTypeManaged;
}

typedef cudaError_t (*RunFn)(const lbm::OpArgs&);
const RunFn kRunNoAlloc[7] = {lbm::run_op_q4, lbm::run_op_q5, lbm::run_op_q9, lbm::run_op_q13,
                              lbm::run_op_q17, lbm::run_op_q21, lbm::run_op_q37};

}  // namespace

extern "C" int32_t lbm_reduce_noalloc(int32_t quadrature, const double* weights, double speed_of_sound_squared,
                                      int64_t nx, int64_t ny, const double* f, int32_t kind,
                                      const lbm_analytic* analytic, double* out, void* stream) {
  using namespace lbm;
  if (quadrature < 0 || quadrature > 6 || !weights || !f || !out) return LBM_ERR_INVALID;
  // The node index is a 32-bit integer: lattices of 2^31 nodes or more are rejected.
  // Each factor is bounded first, so the product below cannot wrap.
  if (nx < 1 || ny < 1 || nx >= (int64_t(1) << 31) || ny >= (int64_t(1) << 31) || nx * ny >= (int64_t(1) << 31))
    return LBM_ERR_INVALID;
  int K = 0;
  switch (kind) {
    case LBM_REDUCE_TRACK_ERRORS: K = 16; break;
    case LBM_REDUCE_COMPARE: K = 12; break;
    case LBM_REDUCE_MEAN_VELOCITY: K = 2; break;
    case LBM_REDUCE_CONSERVED: K = 4; break;
    default: return LBM_ERR_UNSUPPORTED;  // VELOCITY_CONVERGENCE keeps state; DENSITY_AT needs no scratch
  }
  if (kind == LBM_REDUCE_TRACK_ERRORS || kind == LBM_REDUCE_COMPARE) {
    if (!analytic || !analytic->on_device) return LBM_ERR_INVALID;
    const double* need[8] = {analytic->rho, analytic->ux, analytic->uy, analytic->p,
                             analytic->sxx, analytic->syx, analytic->sxy, analytic->syy};
    for (int k = 0; k < (kind == LBM_REDUCE_TRACK_ERRORS ? 8 : 4); ++k)
      if (!need[k]) return LBM_ERR_INVALID;
  }
  const int64_t n = nx * ny;
  const int nblocks = (int)std::min<int64_t>((n + kRedThreads - 1) / kRedThreads, kNoAllocBlocks);
  if ((int64_t)nblocks * K > kNoAllocSlots) return LBM_ERR_INVALID;

  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    (void)cudaGetLastError();
    return LBM_ERR_CUDA;
  }
  if (!on_device(f, dev) || !on_device(out, dev)) return LBM_ERR_INVALID;
  if (kind == LBM_REDUCE_TRACK_ERRORS || kind == LBM_REDUCE_COMPARE) {
    const double* fields[8] = {analytic->rho, analytic->ux, analytic->uy, analytic->p,
                               analytic->sxx, analytic->syx, analytic->sxy, analytic->syy};
    for (int k = 0; k < (kind == LBM_REDUCE_TRACK_ERRORS ? 8 : 4); ++k)
      if (!on_device(fields[k], dev)) return LBM_ERR_INVALID;
  }

  double* scratch = nullptr;
  if (scratch_address(&scratch) != cudaSuccess) {
    (void)cudaGetLastError();  // reported as the status: not left for a later launch check to find
    return LBM_ERR_CUDA;
  }

  // Kernel parameters on the stack: only the fields the reductions read are set.
  StepParams<double> p{};
  p.nx = (int)nx;
  p.ny = (int)ny;
  p.n = n;
  ReduceArgs r{};
  r.kind = kind;
  for (int i = 0; i < LBM_MAX_Q; ++i) r.w[i] = 0.0;
  const int Q[7] = {4, 5, 9, 13, 17, 25, 37};
  for (int i = 0; i < Q[quadrature]; ++i) r.w[i] = weights[i];
  r.cs = speed_of_sound_squared;
  r.q_low_order = (quadrature == LBM_D2Q4 || quadrature == LBM_D2Q5) ? 1 : 0;
  if (analytic) {
    r.rho_a = analytic->rho;
    r.ux_a = analytic->ux;
    r.uy_a = analytic->uy;
    r.p_a = analytic->p;
    r.sxx_a = analytic->sxx;
    r.syx_a = analytic->syx;
    r.sxy_a = analytic->sxy;
    r.syy_a = analytic->syy;
    r.tau = analytic->tau;
    r.u_max = analytic->u_max;
    r.area = analytic->area;
  }
  OpArgs a;
  a.op = OP_REDUCE;
  a.storage = LBM_STORE_F64;
  a.pull = false;  // f is the observed state (f_stream) itself
  a.src = f;
  a.pd = &p;
  a.red = &r;
  a.red_k = K;
  a.partial = scratch;
  a.nblocks = nblocks;
  a.out = out;
  a.stream = static_cast<cudaStream_t>(stream);
  return kRunNoAlloc[quadrature](a) == cudaSuccess ? LBM_OK : LBM_ERR_CUDA;
}
