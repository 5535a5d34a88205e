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

#include "lbm_step.cuh"

namespace lbm {

constexpr int kBatchMax = 65536;  // members per batch

template <class CT>
struct BatchMember {
  StepParams<CT> p;
  void* buf0;            // member buffers (the member context owns them)
  void* buf1;
  int qid;
  int cur0;              // buffer holding the member's state when the batch starts
  int phase0;            // 0: f_stream resident (first step collides only), 1: post-collision
  long long steps;       // steps this member takes
  long long block_start; // first global block index of the member (prefix sum)
};

template <class L, class S, int COLL>
__device__ __forceinline__ void batch_node_step(const StepParams<typename S::C>& p, const typename S::T* src,
                                                typename S::T* dst, int x, int y, bool local) {
  using CT = typename S::C;
  const int node = y * p.nx + x;
  CT v[L::Q];
  if (local) load_local<L, S>(p, src, node, v);
  else load_streamed<L, S>(p, src, x, y, v);
  collide_node<L, S, COLL>(p, x, y, v);
#pragma unroll
  for (int i = 0; i < L::Q; ++i) S::st(dst + (size_t)i * p.n + node, v[i]);
}

// One global step t over the first `nactive` members of one velocity set (members of other sets
// run in their own launch of the same step).  A block covers kBlockX consecutive nodes (x
// fastest) of one member, so lattices of a few nodes use a few threads, not a row of blocks.
template <class L, class S, int COLL>
__global__ void __launch_bounds__(kBlockX) batch_step_kernel(const BatchMember<typename S::C>* __restrict__ members,
                                                             int nactive, long long t) {
  using T = typename S::T;
  const long long b = blockIdx.x;
  int lo = 0, hi = nactive - 1;
  while (lo < hi) {  // last member whose block_start <= b
    const int mid = (lo + hi + 1) >> 1;
    if (members[mid].block_start <= b) lo = mid;
    else hi = mid - 1;
  }
  const BatchMember<typename S::C>& m = members[lo];
  const StepParams<typename S::C>& p = m.p;
  const long long node = (b - m.block_start) * kBlockX + threadIdx.x;
  if (node >= p.n) return;
  const int y = (int)(node / p.nx);
  const int x = (int)(node - (long long)y * p.nx);
  const int parity = (int)((m.cur0 + t) & 1);
  const T* src = static_cast<const T*>(parity ? m.buf1 : m.buf0);
  T* dst = static_cast<T*>(parity ? m.buf0 : m.buf1);
  const bool local = (t == 0) && (m.phase0 == 0);
  batch_node_step<L, S, COLL>(p, src, dst, x, y, local);
}

}  // namespace lbm
