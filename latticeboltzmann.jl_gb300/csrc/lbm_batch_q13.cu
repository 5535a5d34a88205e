// Batched step and reduction kernels for the D2Q13 velocity set (own translation unit, so the
// velocity sets compile in parallel).
#include "lbm_resident.cuh"

namespace lbm {
LBM_BATCH_INSTANTIATE(q13, D2Q13)
}  // namespace lbm
LBM_RESIDENT_INSTANTIATE(q13, D2Q13)
