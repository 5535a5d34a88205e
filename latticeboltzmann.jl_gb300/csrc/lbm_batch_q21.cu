// Batched step and reduction kernels for the D2Q21 velocity set (own translation unit, so the
// velocity sets compile in parallel).
#include "lbm_resident.cuh"

namespace lbm {
LBM_BATCH_INSTANTIATE(q21, D2Q21)
}  // namespace lbm
LBM_RESIDENT_INSTANTIATE(q21, D2Q21)
