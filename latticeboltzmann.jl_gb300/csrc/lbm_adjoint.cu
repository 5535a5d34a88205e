// lbm_adjoint.cu -- instantiations and launcher of the adjoint kernels (lbm_adjoint.cuh) for
// D2Q9 and D2Q13 (second-order equilibria), SRT, TRT and MRT, FP64 and FP32-deviation storage.
#include "lbm_adjoint.cuh"

namespace lbm {

enum AdjOp { ADJ_INIT = 0, ADJ_LOSS = 1, ADJ_STEP = 2, ADJ_U0 = 3 };

template <class L, class S>
cudaError_t adj_run(int op, int coll, const StepParams<typename S::C>& p, AdjArgs a, const void* src, int pull,
                    const void* lam_next, void* lam_out, double* slots, int nblocks, const double* u0,
                    const double* ut, double* grad, cudaStream_t s) {
  using T = typename S::T;
  switch (op) {
    case ADJ_INIT:
      adj_init_kernel<L, S><<<nblocks, kAdjThreads, 0, s>>>(p, u0, static_cast<T*>(lam_out));
      break;
    case ADJ_LOSS:
      adj_loss_kernel<L, S><<<nblocks, kAdjThreads, 0, s>>>(p, static_cast<const T*>(src), ut, static_cast<T*>(lam_out),
                                                            slots);
      break;
    case ADJ_STEP:
      if (coll == LBM_TRT)
        launch_after_prior(adj_step_kernel<L, S, LBM_TRT>, dim3(nblocks), dim3(kAdjThreads), s, p, a,
                           static_cast<const T*>(src), pull, static_cast<const T*>(lam_next),
                           static_cast<T*>(lam_out), slots);
      else if (coll == LBM_MRT)
        launch_after_prior(adj_step_kernel<L, S, LBM_MRT>, dim3(nblocks), dim3(kAdjThreads), s, p, a,
                           static_cast<const T*>(src), pull, static_cast<const T*>(lam_next),
                           static_cast<T*>(lam_out), slots);
      else
        launch_after_prior(adj_step_kernel<L, S, LBM_SRT>, dim3(nblocks), dim3(kAdjThreads), s, p, a,
                           static_cast<const T*>(src), pull, static_cast<const T*>(lam_next),
                           static_cast<T*>(lam_out), slots);
      break;
    case ADJ_U0:
      adj_u0_kernel<L, S><<<nblocks, kAdjThreads, 0, s>>>(p, u0, static_cast<const T*>(lam_next), grad);
      break;
    default:
      return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t adj_launch(int op, int qid, int storage, int coll, const void* params, AdjArgs a, const void* src, int pull,
                       const void* lam_next, void* lam_out, double* slots, int nblocks, const double* u0,
                       const double* ut, double* grad, cudaStream_t s) {
  if (storage == LBM_STORE_F64) {
    const auto& p = *static_cast<const StepParams<double>*>(params);
    if (qid == LBM_D2Q9) return adj_run<D2Q9, F64>(op, coll, p, a, src, pull, lam_next, lam_out, slots, nblocks, u0, ut, grad, s);
    if (qid == LBM_D2Q13) return adj_run<D2Q13, F64>(op, coll, p, a, src, pull, lam_next, lam_out, slots, nblocks, u0, ut, grad, s);
  } else if (storage == LBM_STORE_F32_DEV) {
    const auto& p = *static_cast<const StepParams<float>*>(params);
    if (qid == LBM_D2Q9) return adj_run<D2Q9, F32Dev>(op, coll, p, a, src, pull, lam_next, lam_out, slots, nblocks, u0, ut, grad, s);
    if (qid == LBM_D2Q13) return adj_run<D2Q13, F32Dev>(op, coll, p, a, src, pull, lam_next, lam_out, slots, nblocks, u0, ut, grad, s);
  }
  return cudaErrorInvalidValue;
}

cudaError_t adj_finish(const double* slots, int nblocks, int k, double* out, cudaStream_t s) {
  if (k == 1) adj_finish_kernel<1><<<1, 32, 0, s>>>(slots, nblocks, out);
  else adj_finish_kernel<kAdjParams><<<1, 32, 0, s>>>(slots, nblocks, out);
  return cudaGetLastError();
}

}  // namespace lbm
