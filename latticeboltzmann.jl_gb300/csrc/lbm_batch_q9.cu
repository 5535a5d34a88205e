// Batched step and reduction kernels for the D2Q9 velocity set (own translation unit, so the
// velocity sets compile in parallel).
#include "lbm_resident.cuh"

namespace lbm {
LBM_BATCH_INSTANTIATE(q9, D2Q9)
}  // namespace lbm
LBM_RESIDENT_INSTANTIATE(q9, D2Q9)
