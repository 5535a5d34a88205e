// Kernel instantiations for the D2Q21 velocity set with DF64Dev storage.
#include "lbm_ops.cuh"

namespace lbm {
cudaError_t run_op_q21_df64(const OpArgs& a) { return run_op_s<D2Q21, DF64Dev>(a, *a.px); }
}  // namespace lbm
