// lbm_batch.cuh -- many lattices of uneven size and velocity set advanced by one kernel per
// global time step, all steps captured in one CUDA graph.
//
// A convergence study (the reference runs one `simulate` per (N, q, τ) point, e.g.
// examples/notebooks/taylor_green_vortex.ipynb cell 3) is a set of independent lattices whose
// step counts grow like N².  Launched one after another, the small lattices cannot fill the GPU
// and each of their steps costs a kernel launch.  Here every launch covers the blocks of every
// lattice still running at that global step: lattices are ordered by step count (descending),
// so the running set is a prefix and so is its block list; a block finds its lattice by binary
// search over the prefix sums of block counts.  Each member keeps its own buffers, parameters
// and ping-pong parity; the graph holds one kernel node per global step.
#pragma once

#include "lbm_reduce.cuh"

namespace lbm {

constexpr int kBatchMax = 65536;  // members per batch

// What stays fixed for a member over the batch's life: parameters and buffers.
template <class CT>
struct BatchStatic {
  StepParams<CT> p;
  void* buf0;  // member buffers (the member context owns them)
  void* buf1;
};

// Per call, in launch order (members grouped by velocity set, descending step count).
struct BatchDyn {
  long long block_start;  // first block of the member within its group (prefix sum)
  long long steps;        // steps this member takes (stepping) / its block count (reductions)
  int member;             // index into the static array
  int cur0;               // buffer holding the member's state when the call starts
  int phase0;             // 0: f_stream resident (no pull, a first step collides only), 1: post-collision
  int pad;
  long long t0;           // the member's time index at the first step of the call
  double dt;              // its time step: step t of the call runs at physical time (t0 + t) dt
};

// Last member of the first n whose block_start <= b (block_start is ascending).
__device__ __forceinline__ int batch_find(const BatchDyn* __restrict__ dyn, int n, long long b) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (dyn[mid].block_start <= b) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

template <class L, class S, int COLL, class TimeFn>
__device__ __forceinline__ void batch_node_step(const StepParams<typename S::C>& p, const typename S::T* src,
                                                typename S::T* dst, int x, int y, bool local, TimeFn&& time) {
  using CT = typename S::C;
  const int node = y * p.nx + x;
  CT v[L::Q];
  if (local) load_local<L, S>(p, src, node, v);
  else load_streamed<L, S>(p, src, x, y, v);
  collide_node<L, S, COLL>(p, x, y, v, time);
#pragma unroll
  for (int i = 0; i < L::Q; ++i) S::st(dst + plane_off(p, i) + node, v[i]);
}

// Nodes per block of the batched step: 32 for FP64 storage, whose steps are bound by the FP64 pipe
// (two instructions per SM per clock), so that a lattice of a few hundred nodes spreads over as
// many SMs as it has warps instead of loading two or three (the 28-run shear-wave study's graph:
// 0.071 s instead of 0.075 s); kBlockX for the other storages.
constexpr int batch_block_nodes(int storage) { return storage == LBM_STORE_F64 ? 32 : kBlockX; }

// One global step t over the first `nactive` members of one velocity set (members of other sets
// run in their own launch of the same step).  A block covers NB consecutive nodes (x
// fastest) of one member: a lattice of a few nodes takes one block, so the launch keeps one
// block per small member in flight (packing several small members into one block leaves fewer
// warps to hide the latency of a step that is pure latency at this size; measured slower).
template <class L, class S, int COLL, int NB = batch_block_nodes(S::id)>
__global__ void __launch_bounds__(NB) batch_step_kernel(const BatchStatic<typename S::C>* __restrict__ statics,
                                                             const BatchDyn* __restrict__ dyn, int nactive,
                                                             long long t) {
  using T = typename S::T;
  wait_prior_grid();
  const long long b = blockIdx.x;
  const BatchDyn& d = dyn[batch_find(dyn, nactive, b)];
  const BatchStatic<typename S::C>& m = statics[d.member];
  const StepParams<typename S::C>& p = m.p;
  const long long node = (b - d.block_start) * NB + threadIdx.x;
  if (node >= p.n) return;
  const int y = (int)node / p.nx;
  const int x = (int)node - y * p.nx;
  const int parity = (int)((d.cur0 + t) & 1);
  const T* src = static_cast<const T*>(parity ? m.buf1 : m.buf0);
  T* dst = static_cast<T*>(parity ? m.buf0 : m.buf1);
  const bool local = (t == 0) && (d.phase0 == 0);
  batch_node_step<L, S, COLL>(p, src, dst, x, y, local, [&] { return (double)(d.t0 + t) * d.dt; });
}

// Reductions of many members in one launch: member d.member owns d.steps consecutive blocks
// (from d.block_start), each block writes one partial of K sums, and batch_reduce_finish adds a
// member's partials in block order (deterministic).  The observed state is pulled (with the
// boundary rules) when the member holds its post-collision array.
template <class L, class S, int K>
__global__ void __launch_bounds__(kRedThreads) batch_reduce_kernel(const BatchStatic<typename S::C>* __restrict__ statics,
                                                                   const ReduceArgs* __restrict__ args,
                                                                   const BatchDyn* __restrict__ dyn, int nmem,
                                                                   double* __restrict__ partial) {
  using T = typename S::T;
  const long long b = blockIdx.x;
  const BatchDyn& d = dyn[batch_find(dyn, nmem, b)];
  const BatchStatic<typename S::C>& m = statics[d.member];
  const ReduceArgs& r = args[d.member];
  const T* src = static_cast<const T*>(d.cur0 ? m.buf1 : m.buf0);
  double acc[K];
#pragma unroll
  for (int k = 0; k < K; ++k) acc[k] = 0.0;
  const long long first = (b - d.block_start) * kRedThreads + threadIdx.x;
  const long long stride = d.steps * kRedThreads;
  NodeWalk w(first, stride, m.p.nx);
  for (long long node = first; node < m.p.n; node += stride, w.advance()) {
    if (d.phase0) reduce_node<L, S, true, K>(m.p, r, src, w.x, w.y, node, acc);
    else reduce_node<L, S, false, K>(m.p, r, src, w.x, w.y, node, acc);
  }
  block_reduce_store<K>(acc, partial);
}

template <int K>
__global__ void batch_reduce_finish(const BatchDyn* __restrict__ dyn, int nmem, const double* __restrict__ partial,
                                    long long part_base, double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nmem * K) return;
  const int r = i / K, k = i - r * K;
  const BatchDyn& d = dyn[r];
  double s = 0.0;
  for (long long bb = 0; bb < d.steps; ++bb) s += partial[(size_t)(part_base + d.block_start + bb) * K + k];
  out[(size_t)d.member * kRedMaxK + k] = s;
}

// ---- launchers, instantiated per velocity set in lbm_batch_q*.cu ----------------------------

template <class L, class S>
cudaError_t batch_step_s(int coll, const void* statics, const BatchDyn* dyn, int nactive, long long blocks,
                         long long t, cudaStream_t s) {
  const dim3 g((unsigned)blocks);
  const auto* m = static_cast<const BatchStatic<typename S::C>*>(statics);
  switch (coll) {
    case LBM_SRT: launch_after_prior(batch_step_kernel<L, S, LBM_SRT>, g, batch_block_nodes(S::id), s, m, dyn, nactive, t); break;
    case LBM_TRT: launch_after_prior(batch_step_kernel<L, S, LBM_TRT>, g, batch_block_nodes(S::id), s, m, dyn, nactive, t); break;
    case LBM_MRT: launch_after_prior(batch_step_kernel<L, S, LBM_MRT>, g, batch_block_nodes(S::id), s, m, dyn, nactive, t); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

// One global step t for the first `nactive` members (in launch order) of velocity set L.
template <class L>
cudaError_t batch_launch_set(int storage, int coll, const void* statics, const BatchDyn* dyn, int nactive,
                             long long blocks, long long t, cudaStream_t s) {
  if (blocks <= 0) return cudaSuccess;
  switch (storage) {
    case LBM_STORE_F64: return batch_step_s<L, F64>(coll, statics, dyn, nactive, blocks, t, s);
    case LBM_STORE_DF64_DEV: return batch_step_s<L, DF64Dev>(coll, statics, dyn, nactive, blocks, t, s);
    case LBM_STORE_F32_DEV: return batch_step_s<L, F32Dev>(coll, statics, dyn, nactive, blocks, t, s);
    default: return cudaErrorInvalidValue;
  }
}

template <class L, class S>
cudaError_t batch_reduce_s(int K, const void* statics, const ReduceArgs* args, const BatchDyn* dyn, int nmem,
                           long long blocks, double* partial, long long part_base, double* out, cudaStream_t s) {
  const auto* m = static_cast<const BatchStatic<typename S::C>*>(statics);
  double* part = partial + (size_t)part_base * K;
  const int fin_threads = 128, fin_blocks = (nmem * K + fin_threads - 1) / fin_threads;
  switch (K) {
    case 2:
      batch_reduce_kernel<L, S, 2><<<(unsigned)blocks, kRedThreads, 0, s>>>(m, args, dyn, nmem, part);
      batch_reduce_finish<2><<<fin_blocks, fin_threads, 0, s>>>(dyn, nmem, partial, part_base, out);
      break;
    case 3:
      batch_reduce_kernel<L, S, 3><<<(unsigned)blocks, kRedThreads, 0, s>>>(m, args, dyn, nmem, part);
      batch_reduce_finish<3><<<fin_blocks, fin_threads, 0, s>>>(dyn, nmem, partial, part_base, out);
      break;
    case 4:
      batch_reduce_kernel<L, S, 4><<<(unsigned)blocks, kRedThreads, 0, s>>>(m, args, dyn, nmem, part);
      batch_reduce_finish<4><<<fin_blocks, fin_threads, 0, s>>>(dyn, nmem, partial, part_base, out);
      break;
    case 12:
      batch_reduce_kernel<L, S, 12><<<(unsigned)blocks, kRedThreads, 0, s>>>(m, args, dyn, nmem, part);
      batch_reduce_finish<12><<<fin_blocks, fin_threads, 0, s>>>(dyn, nmem, partial, part_base, out);
      break;
    case 16:
      batch_reduce_kernel<L, S, 16><<<(unsigned)blocks, kRedThreads, 0, s>>>(m, args, dyn, nmem, part);
      batch_reduce_finish<16><<<fin_blocks, fin_threads, 0, s>>>(dyn, nmem, partial, part_base, out);
      break;
    default:
      return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

// Reductions of the `nmem` members (in launch order) of velocity set L: partial sums from block
// part_base on, one row of kRedMaxK doubles per member (by static index) in `out`.
template <class L>
cudaError_t batch_reduce_set(int storage, int K, const void* statics, const ReduceArgs* args, const BatchDyn* dyn,
                             int nmem, long long blocks, double* partial, long long part_base, double* out,
                             cudaStream_t s) {
  if (blocks <= 0 || nmem <= 0) return cudaSuccess;
  switch (storage) {
    case LBM_STORE_F64: return batch_reduce_s<L, F64>(K, statics, args, dyn, nmem, blocks, partial, part_base, out, s);
    case LBM_STORE_DF64_DEV:
      return batch_reduce_s<L, DF64Dev>(K, statics, args, dyn, nmem, blocks, partial, part_base, out, s);
    case LBM_STORE_F32_DEV:
      return batch_reduce_s<L, F32Dev>(K, statics, args, dyn, nmem, blocks, partial, part_base, out, s);
    default: return cudaErrorInvalidValue;
  }
}

#define LBM_BATCH_INSTANTIATE(NAME, LAT)                                                                         \
  cudaError_t batch_launch_##NAME(int storage, int coll, const void* statics, const BatchDyn* dyn, int nactive, \
                                  long long blocks, long long t, cudaStream_t s) {                              \
    return batch_launch_set<LAT>(storage, coll, statics, dyn, nactive, blocks, t, s);                           \
  }                                                                                                             \
  cudaError_t batch_reduce_##NAME(int storage, int K, const void* statics, const ReduceArgs* args,              \
                                  const BatchDyn* dyn, int nmem, long long blocks, double* partial,             \
                                  long long part_base, double* out, cudaStream_t s) {                           \
    return batch_reduce_set<LAT>(storage, K, statics, args, dyn, nmem, blocks, partial, part_base, out, s);     \
  }

}  // namespace lbm
