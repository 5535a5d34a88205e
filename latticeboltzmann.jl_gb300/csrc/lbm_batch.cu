// lbm_batch.cu -- instantiation and launch of the batched step kernel (lbm_batch.cuh).
#include "lbm_batch.cuh"

namespace lbm {

template <class S, int COLL>
cudaError_t batch_launch_s(int qid, const void* members, int nactive, long long blocks, long long t, cudaStream_t s) {
  const dim3 g((unsigned)blocks);
  const auto* m = static_cast<const BatchMember<typename S::C>*>(members);
  switch (qid) {
    case LBM_D2Q4: batch_step_kernel<D2Q4, S, COLL><<<g, kBlockX, 0, s>>>(m, nactive, t); break;
    case LBM_D2Q5: batch_step_kernel<D2Q5, S, COLL><<<g, kBlockX, 0, s>>>(m, nactive, t); break;
    case LBM_D2Q9: batch_step_kernel<D2Q9, S, COLL><<<g, kBlockX, 0, s>>>(m, nactive, t); break;
    case LBM_D2Q13: batch_step_kernel<D2Q13, S, COLL><<<g, kBlockX, 0, s>>>(m, nactive, t); break;
    case LBM_D2Q17: batch_step_kernel<D2Q17, S, COLL><<<g, kBlockX, 0, s>>>(m, nactive, t); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

// Launch one global step for the members of one velocity set: `members` points at that set's
// descriptors (ordered by step count, descending), the first `nactive` are still running and
// cover `blocks` blocks.
cudaError_t batch_launch(int storage, int coll, int qid, const void* members, int nactive, long long blocks,
                         long long t, cudaStream_t s) {
  if (blocks <= 0) return cudaSuccess;
  if (storage == LBM_STORE_F64)
    return coll == LBM_TRT ? batch_launch_s<F64, LBM_TRT>(qid, members, nactive, blocks, t, s)
                           : batch_launch_s<F64, LBM_SRT>(qid, members, nactive, blocks, t, s);
  if (storage == LBM_STORE_DF64_DEV)
    return coll == LBM_TRT ? batch_launch_s<DF64Dev, LBM_TRT>(qid, members, nactive, blocks, t, s)
                           : batch_launch_s<DF64Dev, LBM_SRT>(qid, members, nactive, blocks, t, s);
  if (storage == LBM_STORE_F32_DEV)
    return coll == LBM_TRT ? batch_launch_s<F32Dev, LBM_TRT>(qid, members, nactive, blocks, t, s)
                           : batch_launch_s<F32Dev, LBM_SRT>(qid, members, nactive, blocks, t, s);
  return cudaErrorInvalidValue;
}

size_t batch_member_size(int storage) {
  if (storage == LBM_STORE_F64) return sizeof(BatchMember<double>);
  if (storage == LBM_STORE_DF64_DEV) return sizeof(BatchMember<dd>);
  return sizeof(BatchMember<float>);
}

}  // namespace lbm
