// Kernel instantiations for the D2Q17 velocity set (separate translation unit so the
// velocity sets compile in parallel).
#include "lbm_ops.cuh"

namespace lbm {
cudaError_t run_op_q17(const OpArgs& a) { return run_op<D2Q17>(a); }
}  // namespace lbm
