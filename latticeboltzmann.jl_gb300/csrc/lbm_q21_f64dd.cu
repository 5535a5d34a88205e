// Kernel instantiations for the D2Q21 velocity set with F64DD storage.
#include "lbm_ops.cuh"

namespace lbm {
cudaError_t run_op_q21_f64dd(const OpArgs& a) { return run_op_s<D2Q21, F64DD>(a, *a.px); }
}  // namespace lbm
