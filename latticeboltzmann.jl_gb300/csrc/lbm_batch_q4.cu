// Batched step and reduction kernels for the D2Q4 velocity set (own translation unit, so the
// velocity sets compile in parallel).
#include "lbm_resident.cuh"

namespace lbm {
LBM_BATCH_INSTANTIATE(q4, D2Q4)
}  // namespace lbm
LBM_RESIDENT_INSTANTIATE(q4, D2Q4)
