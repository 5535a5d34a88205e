// Kernel instantiations for the D2Q37 velocity set with F32DevSR storage.
#include "lbm_ops.cuh"

namespace lbm {
cudaError_t run_op_q37_f32sr(const OpArgs& a) { return run_op_s<D2Q37, F32DevSR>(a, *a.px); }
}  // namespace lbm
