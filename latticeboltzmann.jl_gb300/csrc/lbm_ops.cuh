// lbm_ops.cuh -- kernel launch table, one instantiation per velocity set (lbm_q*.cu), so
// that the velocity sets compile as separate translation units in parallel.
#pragma once

#include "lbm_reduce.cuh"

namespace lbm {

enum Op {
  OP_COLLIDE = 0,    // collide only (local)                      step_kernel MODE 0
  OP_FUSED = 1,      // pull + BCs + collide                      step_kernel MODE 1
  OP_STREAM_BC = 2,  // pull + BCs (materialise f_stream)         step_kernel MODE 2
  OP_STREAM = 3,     // periodic pull only (stream!)              step_kernel MODE 2, no BCs
  OP_APPLY_BC = 4,   // apply!(bcs) in place, FP64 arrays
  OP_REDUCE = 5,     // reductions (+ finish)
  OP_MACRO = 6,      // ρ, u planes
  OP_WIDEN = 7,      // observed populations -> FP64 planes
  OP_NARROW = 8,     // FP64 planes -> storage
  OP_NODE_DENSITY = 9,  // density of node (node_x, node_y)
  OP_INIT_FIELDS = 10   // initial populations from macroscopic planes
};

struct OpArgs {
  int op = 0, storage = 0, coll = 0;
  bool pull = false;                 // reductions / widen / macro: the source is post-collision
  const void* src = nullptr;
  void* dst = nullptr;
  const StepParams<double>* pd = nullptr;
  const StepParams<float>* pf = nullptr;
  const StepParams<dd>* px = nullptr;
  const ReduceArgs* red = nullptr;
  int red_k = 0;
  double* partial = nullptr;
  int nblocks = 0;
  double* out = nullptr;
  int node_x = 0, node_y = 0;
  const InitFields* init = nullptr;
  cudaStream_t stream = 0;
};

inline dim3 lattice_grid(int nx, int ny) {
  return dim3((unsigned)((nx + kBlockX - 1) / kBlockX), (unsigned)(ny < 65535 ? ny : 65535));
}

template <class L, class S, int MODE>
inline void launch_step(const OpArgs& a, const StepParams<typename S::C>& p) {
  const dim3 g = lattice_grid(p.nx, p.ny);
  const auto* src = static_cast<const typename S::T*>(a.src);
  auto* dst = static_cast<typename S::T*>(a.dst);
  // SRT / TRT of the deviation storages: two nodes per thread on packed FP32 pairs (even nx).
  // Where the pair kernel's registers would cut the occupancy too far, the one-node kernel stays:
  // D2Q37 in FP32 / FP16 (154 registers against 72, measured 8 % slower), float-float DF64
  // above D2Q17 (D2Q13 and D2Q17 measured 4 % faster as pairs, D2Q21 and D2Q37 no faster), and
  // the other float-float storages (FP32-SR, FP64-DD) above D2Q9.
  constexpr int kPairMaxQ = std::is_same<typename S::C, dd>::value ? (S::id == LBM_STORE_DF64_DEV ? 17 : 9) : 25;
  constexpr bool kPairs = MODE == 1 && S::DEV && L::Q <= kPairMaxQ;
  if constexpr (kPairs) {
    if ((a.coll == LBM_SRT || a.coll == LBM_TRT) && p.nx % 2 == 0) {
      const dim3 g2((unsigned)((p.nx / 2 + kBlockX - 1) / kBlockX), g.y);
      launch_after_prior(step_pair_kernel<L, S>, g2, kBlockX, a.stream, p, src, dst);
      return;
    }
  }
  switch (a.coll) {
    case LBM_SRT: launch_after_prior(step_kernel<L, S, LBM_SRT, MODE>, g, kBlockX, a.stream, p, src, dst); break;
    case LBM_TRT: launch_after_prior(step_kernel<L, S, LBM_TRT, MODE>, g, kBlockX, a.stream, p, src, dst); break;
    case LBM_MRT: launch_after_prior(step_kernel<L, S, LBM_MRT, MODE>, g, kBlockX, a.stream, p, src, dst); break;
    default: launch_after_prior(step_kernel<L, S, LBM_ITERATIVE_INIT, MODE>, g, kBlockX, a.stream, p, src, dst); break;
  }
}

template <class L, class S, bool PULL>
inline void launch_reduce(const OpArgs& a, const StepParams<typename S::C>& p) {
  const auto* src = static_cast<const typename S::T*>(a.src);
  const int nb = a.nblocks;
  switch (a.red_k) {
    case 16:
      reduce_kernel<L, S, PULL, 16><<<nb, kRedThreads, 0, a.stream>>>(p, *a.red, src, a.partial);
      reduce_finish_kernel<16><<<1, 32, 0, a.stream>>>(a.partial, nb, a.out);
      break;
    case 12:
      reduce_kernel<L, S, PULL, 12><<<nb, kRedThreads, 0, a.stream>>>(p, *a.red, src, a.partial);
      reduce_finish_kernel<12><<<1, 32, 0, a.stream>>>(a.partial, nb, a.out);
      break;
    case 4:
      reduce_kernel<L, S, PULL, 4><<<nb, kRedThreads, 0, a.stream>>>(p, *a.red, src, a.partial);
      reduce_finish_kernel<4><<<1, 32, 0, a.stream>>>(a.partial, nb, a.out);
      break;
    case 3:
      reduce_kernel<L, S, PULL, 3><<<nb, kRedThreads, 0, a.stream>>>(p, *a.red, src, a.partial);
      reduce_finish_kernel<3><<<1, 32, 0, a.stream>>>(a.partial, nb, a.out);
      break;
    default:
      reduce_kernel<L, S, PULL, 2><<<nb, kRedThreads, 0, a.stream>>>(p, *a.red, src, a.partial);
      reduce_finish_kernel<2><<<1, 32, 0, a.stream>>>(a.partial, nb, a.out);
      break;
  }
}

template <class L, class S>
inline cudaError_t run_op_s(const OpArgs& a, const StepParams<typename S::C>& p) {
  const dim3 g = lattice_grid(p.nx, p.ny);
  const auto* src = static_cast<const typename S::T*>(a.src);
  switch (a.op) {
    case OP_COLLIDE: launch_step<L, S, 0>(a, p); break;
    case OP_FUSED: launch_step<L, S, 1>(a, p); break;
    case OP_STREAM_BC:
      step_kernel<L, S, LBM_SRT, 2><<<g, kBlockX, 0, a.stream>>>(p, src, static_cast<typename S::T*>(a.dst));
      break;
    case OP_STREAM: {
      StepParams<typename S::C> q = p;
      q.nbc = 0;
      step_kernel<L, S, LBM_SRT, 2><<<g, kBlockX, 0, a.stream>>>(q, src, static_cast<typename S::T*>(a.dst));
      break;
    }
    case OP_APPLY_BC:
      if constexpr (S::id == LBM_STORE_F64)
        apply_bcs_kernel<L><<<g, kBlockX, 0, a.stream>>>(p, static_cast<double*>(a.dst),
                                                         static_cast<const double*>(a.src));
      else
        return cudaErrorInvalidValue;
      break;
    case OP_REDUCE:
      if (a.pull) launch_reduce<L, S, true>(a, p);
      else launch_reduce<L, S, false>(a, p);
      break;
    case OP_MACRO:
      if (a.pull) macro_kernel<L, S, true><<<g, kBlockX, 0, a.stream>>>(p, *a.red, src, static_cast<double*>(a.dst));
      else macro_kernel<L, S, false><<<g, kBlockX, 0, a.stream>>>(p, *a.red, src, static_cast<double*>(a.dst));
      break;
    case OP_WIDEN:
      if (a.pull) widen_kernel<L, S, true><<<g, kBlockX, 0, a.stream>>>(p, *a.red, src, static_cast<double*>(a.dst));
      else widen_kernel<L, S, false><<<g, kBlockX, 0, a.stream>>>(p, *a.red, src, static_cast<double*>(a.dst));
      break;
    case OP_NARROW:
      narrow_kernel<L, S><<<g, kBlockX, 0, a.stream>>>(p, *a.red, static_cast<const double*>(a.src),
                                                       static_cast<typename S::T*>(a.dst));
      break;
    case OP_INIT_FIELDS:
      init_fields_kernel<L, S><<<g, kBlockX, 0, a.stream>>>(p, *a.red, *a.init, static_cast<typename S::T*>(a.dst));
      break;
    case OP_NODE_DENSITY:
      if (a.pull)
        node_density_kernel<L, S, true><<<1, 32, 0, a.stream>>>(p, *a.red, src, a.node_x, a.node_y, a.out);
      else
        node_density_kernel<L, S, false><<<1, 32, 0, a.stream>>>(p, *a.red, src, a.node_x, a.node_y, a.out);
      break;
    default:
      return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

template <class L>
cudaError_t run_op(const OpArgs& a) {
  switch (a.storage) {
    case LBM_STORE_F64: return run_op_s<L, F64>(a, *a.pd);
    case LBM_STORE_F32_DEV: return run_op_s<L, F32Dev>(a, *a.pf);
    case LBM_STORE_F16_DEV: return run_op_s<L, F16Dev>(a, *a.pf);
    case LBM_STORE_DF64_DEV: return run_op_s<L, DF64Dev>(a, *a.px);
    case LBM_STORE_F32_DEV_SR: return run_op_s<L, F32DevSR>(a, *a.px);
    case LBM_STORE_F64_DD: return run_op_s<L, F64DD>(a, *a.px);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t run_op_q4(const OpArgs& a);
cudaError_t run_op_q5(const OpArgs& a);
cudaError_t run_op_q9(const OpArgs& a);
cudaError_t run_op_q13(const OpArgs& a);
cudaError_t run_op_q17(const OpArgs& a);
cudaError_t run_op_q21(const OpArgs& a);
cudaError_t run_op_q37(const OpArgs& a);

}  // namespace lbm
