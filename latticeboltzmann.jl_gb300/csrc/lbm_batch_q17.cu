// Batched step and reduction kernels for the D2Q17 velocity set (own translation unit, so the
// velocity sets compile in parallel).
#include "lbm_batch.cuh"

namespace lbm {
LBM_BATCH_INSTANTIATE(q17, D2Q17)
}  // namespace lbm
