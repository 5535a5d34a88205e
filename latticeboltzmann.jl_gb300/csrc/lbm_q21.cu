// Kernel dispatch for the D2Q21 velocity set; its instantiations are split by storage
// (lbm_q21_*.cu) so that they compile in parallel.
#include "lbm_ops.cuh"

namespace lbm {
cudaError_t run_op_q21_f64(const OpArgs& a);
cudaError_t run_op_q21_df64(const OpArgs& a);
cudaError_t run_op_q21_f32(const OpArgs& a);
cudaError_t run_op_q21_f16(const OpArgs& a);
cudaError_t run_op_q21_f32sr(const OpArgs& a);
cudaError_t run_op_q21_f64dd(const OpArgs& a);

cudaError_t run_op_q21(const OpArgs& a) {
  switch (a.storage) {
    case LBM_STORE_F64: return run_op_q21_f64(a);
    case LBM_STORE_DF64_DEV: return run_op_q21_df64(a);
    case LBM_STORE_F32_DEV: return run_op_q21_f32(a);
    case LBM_STORE_F16_DEV: return run_op_q21_f16(a);
    case LBM_STORE_F32_DEV_SR: return run_op_q21_f32sr(a);
    case LBM_STORE_F64_DD: return run_op_q21_f64dd(a);
    default: return cudaErrorInvalidValue;
  }
}
}  // namespace lbm
