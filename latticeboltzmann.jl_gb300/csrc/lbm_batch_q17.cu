// Batched step and reduction kernels for the D2Q17 velocity set (own translation unit, so the
// velocity sets compile in parallel).
#include "lbm_resident.cuh"

namespace lbm {
LBM_BATCH_INSTANTIATE(q17, D2Q17)
}  // namespace lbm
LBM_RESIDENT_INSTANTIATE(q17, D2Q17)
