// Kernel instantiations for the D2Q37 velocity set with F16Dev storage.
#include "lbm_ops.cuh"

namespace lbm {
cudaError_t run_op_q37_f16(const OpArgs& a) { return run_op_s<D2Q37, F16Dev>(a, *a.pf); }
}  // namespace lbm
