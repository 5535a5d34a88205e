// Kernel instantiations for the D2Q21 velocity set with F16Dev storage.
#include "lbm_ops.cuh"

namespace lbm {
cudaError_t run_op_q21_f16(const OpArgs& a) { return run_op_s<D2Q21, F16Dev>(a, *a.pf); }
}  // namespace lbm
