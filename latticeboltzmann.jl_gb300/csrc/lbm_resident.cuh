// lbm_resident.cuh -- block-resident batched stepping: a small member of a batch takes all of its
// steps of a call inside ONE kernel launch, its populations held in shared memory.
//
// The graph path (lbm_batch.cuh) issues one kernel per global step; for members of a few dozen to
// a few thousand nodes each of those kernels is pure launch and scheduling latency (~2.4 us per
// graph node, whatever the kernel does).  Here a member gets a thread-block cluster of C CTAs
// (C = 1, 2, 4 or 8, one CTA per SM) that stays resident for the whole call:
//   - CTA r of the cluster owns the member's nodes [r*chunk, min(n, (r+1)*chunk)) (node index
//     y*nx + x, chunk = ceil(n / C)) and holds their Q populations, in both ping-pong buffers,
//     in its own shared memory (plane i of a buffer at i*stride, stride >= chunk);
//   - a step pulls each owned node's populations from the CTA that owns the source node -- its
//     own shared memory, or a neighbour's through distributed shared memory -- applies the
//     boundary rules, collides with the same collide_node as the graph path's batch_step_kernel,
//     and writes the node's new populations to its own other buffer;
//   - a cluster barrier (barrier.cluster arrive.release / wait.acquire, a hardware barrier that
//     every CTA of the cluster reaches the same number of times) separates the steps;
//   - the state is read from and written back to the member's global buffers once per call.
// Spreading a member over C SMs divides its per-step arithmetic (FP64 runs at two instructions
// per SM per clock on this GPU) while the halo reads stay on chip.  The populations and the
// collision arithmetic are the graph path's, so a member gives the same bits either way.
#pragma once

#include <atomic>

#include <cooperative_groups.h>

#include "lbm_batch.cuh"

namespace lbm {

constexpr int kResidentThreads = 256;   // threads per CTA (at most)
constexpr int kResidentMaxCluster = 8;  // CTAs per member (portable cluster size)
// Shared memory a resident member's CTA may plan on: 200 KB, below the opt-in limit per block
// (227 KB on this GPU) with room for the kernel's own static shared memory.
constexpr size_t kResidentMaxSmem = 200 * 1024;

// One member of a resident launch.
struct ResidentDyn {
  int member;      // index into the batch's static array
  int cur0;        // buffer holding the member's state when the call starts
  int phase0;      // 0: f_stream resident (the first step collides only), 1: post-collision
  int chunk;       // nodes per CTA of the member's cluster, ceil(n / C)
  long long steps; // steps of this call (> 0)
  long long t0;    // time index of the first step: step t runs at physical time (t0 + t) dt
  double dt;
};

// Storage traits for populations held in shared memory: the element and compute types of S, read
// with plain (coherent) loads instead of the read-only data path S::ld takes for global memory.
template <class S>
struct SmemStore;
template <>
struct SmemStore<F64> : F64 {
  __device__ __forceinline__ static C ld(const T* p) { return *p; }
};
template <>
struct SmemStore<F32Dev> : F32Dev {
  __device__ __forceinline__ static C ld(const T* p) { return *p; }
};
template <>
struct SmemStore<DF64Dev> : DF64Dev {
  __device__ __forceinline__ static C ld(const T* p) {
    const float2 v = *p;
    return dd(v.x, v.y);
  }
};

// Where population i of member node s lives in the cluster: CTA s / chunk, local node s % chunk.
template <class T>
struct ClusterPlanes {
  T* local;      // this CTA's buffer
  int rank;      // this CTA's rank in the cluster
  int chunk;     // nodes per CTA
  int stride;    // plane stride of the buffers
  __device__ __forceinline__ const T* at(int i, int s) const {
    const int owner = (unsigned)s / (unsigned)chunk;
    const int off = s - owner * chunk;
    T* p = local + (size_t)i * stride + off;
    if (owner == rank) return p;
    return cooperative_groups::this_cluster().map_shared_rank(p, (unsigned)owner);
  }
};

// Streamed populations of node (x, y) (owned by this CTA as local node j): the periodic pull of
// stream!, then the boundary conditions in list order, exactly as load_streamed does it on a
// global array (bounce_back.jl:8-72, moving_wall.jl:17-38).
template <class L, class V, class CT>
__device__ __forceinline__ void resident_pull(const StepParams<CT>& p, const ClusterPlanes<typename V::T>& src,
                                              int x, int y, int j, typename V::C* f) {
  int xw[2 * L::R + 1], yo[2 * L::R + 1];
  pull_offsets<L>(p, x, y, xw, yo);
#pragma unroll
  for (int i = 0; i < L::Q; ++i) f[i] = V::ld(src.at(i, yo[L::R + L::cy(i)] + xw[L::R + L::cx(i)]));
  if (p.nbc > 0 && (y < L::R || y >= p.ny - L::R || x < L::R || x >= p.nx - L::R)) {
    const typename V::T* own = src.local + j;
    const int y1 = y + 1, x1 = x + 1;  // the reference's 1-based indices
    for (int b = 0; b < p.nbc; ++b) {
      const BCDev& bc = p.bc[b];
      if (bc.kind == LBM_BOUNCE_BACK) {
        if (x < bc.x_lo || x > bc.x_hi || y < bc.y_lo || y > bc.y_hi) continue;
#pragma unroll
        for (int i = 0; i < L::Q; ++i) {
          const int o = L::opp(i);
          bool hit;
          if (bc.dir == LBM_NORTH) hit = y1 + L::cy(o) > p.ny;
          else if (bc.dir == LBM_SOUTH) hit = y1 + L::cy(o) <= 0;
          else if (bc.dir == LBM_EAST) hit = x1 + L::cx(o) > p.nx;
          else hit = x1 + L::cx(o) <= 0;
          if (hit) f[i] = V::ld(own + (size_t)o * src.stride);
        }
      } else {  // MovingWall{North}: whole top wall, ignores xs / ys
#pragma unroll
        for (int i = 0; i < L::Q; ++i) {
          const int o = L::opp(i);
          if (y1 + L::cy(o) > p.ny) f[i] = V::ld(own + (size_t)o * src.stride) + (typename V::C)bc.add[i];
        }
      }
    }
  }
}

// All steps of one call for the members of one launch (one velocity set, one cluster size):
// member blockIdx.x / C, cluster rank blockIdx.x % C.  Dynamic shared memory: two buffers of Q
// planes of `stride` populations.  Every CTA runs every step and every cluster barrier, including
// CTAs that own no node (members smaller than C), so the barriers always complete.
//
// PARTS > 1 splits each node's SRT / TRT collision over PARTS warps (owns_pop, lbm_step.cuh):
// warp w takes the nodes of group w / PARTS (32 nodes, one per lane) and computes the outputs of
// part w % PARTS, which is the same for the whole warp, so the split costs no divergence.  A
// small member is bound by the latency of one warp's collision (FP64 issues at two lanes per SM
// per clock), and a split shortens that chain to the node-wide sums plus a share of the outputs.
template <class L, class S, int COLL, int PARTS>
__global__ void __launch_bounds__(kResidentThreads) resident_step_kernel(
    const BatchStatic<typename S::C>* __restrict__ statics, const ResidentDyn* __restrict__ dyn, int csize,
    int stride) {
  namespace cg = cooperative_groups;
  using T = typename S::T;
  using CT = typename S::C;
  using V = SmemStore<S>;
  extern __shared__ __align__(16) unsigned char resident_smem[];
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const ResidentDyn d = dyn[blockIdx.x / csize];
  const BatchStatic<CT>& m = statics[d.member];
  const StepParams<CT>& p = m.p;
  T* cur = reinterpret_cast<T*>(resident_smem);      // the state
  T* nxt = cur + (size_t)L::Q * stride;                // the next step's state
  const int n = (int)p.n;
  const int base = rank * d.chunk;
  const int count = max(0, min(n - base, d.chunk));

  // the member's slice of the state into buffer 0
  const T* g = static_cast<const T*>(d.cur0 ? m.buf1 : m.buf0);
  for (int k = threadIdx.x; k < L::Q * count; k += blockDim.x) {
    const int i = k / count, j = k - i * count;
    cur[(size_t)i * stride + j] = g[(size_t)i * n + base + j];
  }
  cluster.sync();

  const int warp = threadIdx.x >> 5;
  const int part = warp % PARTS;                      // the same for every lane of a warp
  const int first = (warp / PARTS) * 32 + (threadIdx.x & 31);
  const int jstep = (blockDim.x / (32 * PARTS)) * 32;  // nodes covered by all groups of the CTA
  for (long long t = 0; t < d.steps; ++t) {
    const ClusterPlanes<T> src{cur, rank, d.chunk, stride};
    T* dst = nxt;
    for (int j = first; j < count; j += jstep) {
      const int node = base + j;
      const int y = node / p.nx;
      const int x = node - y * p.nx;
      CT v[L::Q];
      if (t == 0 && d.phase0 == 0) {
#pragma unroll
        for (int i = 0; i < L::Q; ++i) v[i] = V::ld(cur + (size_t)i * stride + j);
      } else {
        resident_pull<L, V>(p, src, x, y, j, v);
      }
      static_for<0, PARTS>([&](auto P) {
        constexpr int PP = decltype(P)::value;
        if (part == PP) {
          collide_node<L, S, COLL, PARTS, PP>(p, x, y, v, [&] { return (double)(d.t0 + t) * d.dt; });
          static_for<0, L::Q>([&](auto I) {
            constexpr int i = decltype(I)::value;
            if constexpr (owns_pop<L, PARTS, PP>(i)) V::st(dst + (size_t)i * stride + j, v[i]);
          });
        }
      });
    }
    cluster.sync();  // this step's writes visible, and every read of the old buffer done
    nxt = cur;
    cur = dst;
  }

  // the final state into the buffer the member's parity names after d.steps steps
  T* out = static_cast<T*>(((d.cur0 + d.steps) & 1) ? m.buf1 : m.buf0);
  for (int k = threadIdx.x; k < L::Q * count; k += blockDim.x) {
    const int i = k / count, j = k - i * count;
    out[(size_t)i * n + base + j] = cur[(size_t)i * stride + j];
  }
}

// Shared memory of one CTA holding `stride` nodes per plane, both buffers.
template <class L, class S>
constexpr size_t resident_smem_bytes(int stride) {
  return 2 * (size_t)L::Q * (size_t)stride * sizeof(typename S::T);
}

// The largest dynamic shared memory a CTA of `kernel` may use on the current device: the device's
// opt-in limit per block less the kernel's static shared memory.  The kernel's attribute is raised
// to that once per device (an attribute change while the same kernel runs on another stream could
// order the launches), and the result is kept in `allowed` (per device: 0 unknown, else the limit
// + 1), which the caller keeps for this one kernel.
template <class K>
cudaError_t allow_resident_smem(K kernel, std::atomic<long long>* allowed, size_t* limit) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  long long have = allowed[dev].load();
  if (have == 0) {
    int optin = 0;
    cudaFuncAttributes fa{};
    e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, kernel);
    if (e != cudaSuccess) return e;
    const long long lim = (long long)optin - (long long)fa.sharedSizeBytes;
    if (lim <= 0) return cudaErrorInvalidValue;
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lim);
    if (e != cudaSuccess) return e;
    have = lim + 1;
    allowed[dev].store(have);
  }
  *limit = (size_t)(have - 1);
  return cudaSuccess;
}

template <class L, class S, int COLL, int PARTS>
cudaError_t resident_launch_k(const void* statics, const ResidentDyn* dyn, int nmem, int csize, int stride,
                              int threads, size_t smem_min, cudaStream_t s) {
  auto kernel = resident_step_kernel<L, S, COLL, PARTS>;
  static std::atomic<long long> allowed[64];  // this kernel's shared-memory limit per device
  size_t smem = resident_smem_bytes<L, S>(stride);
  if (threads % (32 * PARTS) != 0) return cudaErrorInvalidValue;
  size_t limit = 0;
  cudaError_t e = allow_resident_smem(kernel, allowed, &limit);
  if (e != cudaSuccess) return e;
  if (smem > limit) return cudaErrorInvalidValue;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(nmem * csize));
  cfg.blockDim = dim3((unsigned)threads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)csize;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (smem_min > smem) {  // one CTA per SM, if all of this launch's clusters fit that way at once
    cudaLaunchConfig_t wide = cfg;
    wide.dynamicSmemBytes = smem_min < limit ? smem_min : limit;
    int fit = 0;
    if (cudaOccupancyMaxActiveClusters(&fit, kernel, &wide) == cudaSuccess && fit >= nmem) cfg = wide;
    else (void)cudaGetLastError();
  }
  e = cudaLaunchKernelEx(&cfg, kernel, static_cast<const BatchStatic<typename S::C>*>(statics), dyn, csize, stride);
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

// Splits are built for the pair-form collisions (SRT, TRT) of the FP64-class storages from D2Q9
// up, where one warp's collision chain is long; elsewhere a node's collision stays in one warp.
template <class L, class S>
constexpr bool resident_splits() {
  return (S::id == LBM_STORE_F64 || S::id == LBM_STORE_DF64_DEV) && L::Q >= 9;
}

template <class L, class S, int COLL>
cudaError_t resident_launch_c(const void* statics, const ResidentDyn* dyn, int nmem, int csize, int stride,
                              int threads, int parts, size_t smem_min, cudaStream_t s) {
  if constexpr ((COLL == LBM_SRT || COLL == LBM_TRT) && resident_splits<L, S>()) {
    if (parts == 2) return resident_launch_k<L, S, COLL, 2>(statics, dyn, nmem, csize, stride, threads, smem_min, s);
    if (parts == 4) return resident_launch_k<L, S, COLL, 4>(statics, dyn, nmem, csize, stride, threads, smem_min, s);
  }
  if (parts != 1) return cudaErrorInvalidValue;
  return resident_launch_k<L, S, COLL, 1>(statics, dyn, nmem, csize, stride, threads, smem_min, s);
}

template <class L, class S>
cudaError_t resident_launch_s(int coll, const void* statics, const ResidentDyn* dyn, int nmem, int csize, int stride,
                              int threads, int parts, size_t smem_min, cudaStream_t s) {
  switch (coll) {
    case LBM_SRT: return resident_launch_c<L, S, LBM_SRT>(statics, dyn, nmem, csize, stride, threads, parts, smem_min, s);
    case LBM_TRT: return resident_launch_c<L, S, LBM_TRT>(statics, dyn, nmem, csize, stride, threads, parts, smem_min, s);
    case LBM_MRT: return resident_launch_c<L, S, LBM_MRT>(statics, dyn, nmem, csize, stride, threads, parts, smem_min, s);
    default: return cudaErrorInvalidValue;
  }
}

// One resident launch: `nmem` members of velocity set L, each on a cluster of `csize` CTAs of
// `threads` threads (a multiple of 32 * parts) with `stride` nodes per plane in shared memory, each
// node's collision split over `parts` warps (1, 2 or 4).  A CTA asks for at least `smem_min` bytes
// of shared memory -- more than half an SM's keeps every CTA on an SM of its own -- when the
// device can hold all of the launch's clusters at once that way (cudaOccupancyMaxActiveClusters);
// otherwise it asks for what its populations need.
template <class L>
cudaError_t resident_launch_set(int storage, int coll, const void* statics, const ResidentDyn* dyn, int nmem,
                                int csize, int stride, int threads, int parts, size_t smem_min, cudaStream_t s) {
  if (nmem <= 0) return cudaSuccess;
  if (csize < 1 || csize > kResidentMaxCluster || threads < 32 || threads > kResidentThreads) return cudaErrorInvalidValue;
  switch (storage) {
    case LBM_STORE_F64:
      return resident_launch_s<L, F64>(coll, statics, dyn, nmem, csize, stride, threads, parts, smem_min, s);
    case LBM_STORE_DF64_DEV:
      return resident_launch_s<L, DF64Dev>(coll, statics, dyn, nmem, csize, stride, threads, parts, smem_min, s);
    case LBM_STORE_F32_DEV:
      return resident_launch_s<L, F32Dev>(coll, statics, dyn, nmem, csize, stride, threads, parts, smem_min, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace lbm

#define LBM_RESIDENT_INSTANTIATE(NAME, LAT)                                                                    \
  namespace lbm {                                                                                              \
  cudaError_t resident_launch_##NAME(int storage, int coll, const void* statics, const ResidentDyn* dyn,       \
                                     int nmem, int csize, int stride, int threads, int parts, size_t smem_min, cudaStream_t s) { \
    return resident_launch_set<LAT>(storage, coll, statics, dyn, nmem, csize, stride, threads, parts, smem_min, s);      \
  }                                                                                                            \
  }
