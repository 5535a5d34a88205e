// lbm_batch.cu -- instantiations and launchers of the batched step and reduction kernels
// (lbm_batch.cuh).
#include "lbm_batch.cuh"

namespace lbm {

namespace {

template <class S, int COLL>
cudaError_t step_s(int qid, const void* statics, const BatchDyn* dyn, int nactive, long long blocks, long long t,
                   cudaStream_t s) {
  const dim3 g((unsigned)blocks);
  const auto* m = static_cast<const BatchStatic<typename S::C>*>(statics);
  switch (qid) {
    case LBM_D2Q4: batch_step_kernel<D2Q4, S, COLL><<<g, kBlockX, 0, s>>>(m, dyn, nactive, t); break;
    case LBM_D2Q5: batch_step_kernel<D2Q5, S, COLL><<<g, kBlockX, 0, s>>>(m, dyn, nactive, t); break;
    case LBM_D2Q9: batch_step_kernel<D2Q9, S, COLL><<<g, kBlockX, 0, s>>>(m, dyn, nactive, t); break;
    case LBM_D2Q13: batch_step_kernel<D2Q13, S, COLL><<<g, kBlockX, 0, s>>>(m, dyn, nactive, t); break;
    case LBM_D2Q17: batch_step_kernel<D2Q17, S, COLL><<<g, kBlockX, 0, s>>>(m, dyn, nactive, t); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

template <class L, class S>
cudaError_t reduce_k(int K, const void* statics, const ReduceArgs* args, const BatchDyn* dyn, int nmem,
                     long long blocks, double* partial, long long part_base, double* out, cudaStream_t s) {
  const auto* m = static_cast<const BatchStatic<typename S::C>*>(statics);
  double* part = partial + (size_t)part_base * K;
  const int fin_threads = 128, fin_blocks = (nmem * K + fin_threads - 1) / fin_threads;
  switch (K) {
    case 2:
      batch_reduce_kernel<L, S, 2><<<(unsigned)blocks, kRedThreads, 0, s>>>(m, args, dyn, nmem, part);
      batch_reduce_finish<2><<<fin_blocks, fin_threads, 0, s>>>(dyn, nmem, partial, part_base, out);
      break;
    case 3:
      batch_reduce_kernel<L, S, 3><<<(unsigned)blocks, kRedThreads, 0, s>>>(m, args, dyn, nmem, part);
      batch_reduce_finish<3><<<fin_blocks, fin_threads, 0, s>>>(dyn, nmem, partial, part_base, out);
      break;
    case 4:
      batch_reduce_kernel<L, S, 4><<<(unsigned)blocks, kRedThreads, 0, s>>>(m, args, dyn, nmem, part);
      batch_reduce_finish<4><<<fin_blocks, fin_threads, 0, s>>>(dyn, nmem, partial, part_base, out);
      break;
    default:
      return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

template <class S>
cudaError_t reduce_s(int qid, int K, const void* statics, const ReduceArgs* args, const BatchDyn* dyn, int nmem,
                     long long blocks, double* partial, long long part_base, double* out, cudaStream_t s) {
  switch (qid) {
    case LBM_D2Q4: return reduce_k<D2Q4, S>(K, statics, args, dyn, nmem, blocks, partial, part_base, out, s);
    case LBM_D2Q5: return reduce_k<D2Q5, S>(K, statics, args, dyn, nmem, blocks, partial, part_base, out, s);
    case LBM_D2Q9: return reduce_k<D2Q9, S>(K, statics, args, dyn, nmem, blocks, partial, part_base, out, s);
    case LBM_D2Q13: return reduce_k<D2Q13, S>(K, statics, args, dyn, nmem, blocks, partial, part_base, out, s);
    case LBM_D2Q17: return reduce_k<D2Q17, S>(K, statics, args, dyn, nmem, blocks, partial, part_base, out, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace

// One global step t for the first `nactive` members (in launch order) of one velocity set.
cudaError_t batch_launch(int storage, int coll, int qid, const void* statics, const BatchDyn* dyn, int nactive,
                         long long blocks, long long t, cudaStream_t s) {
  if (blocks <= 0) return cudaSuccess;
  if (storage == LBM_STORE_F64)
    return coll == LBM_TRT ? step_s<F64, LBM_TRT>(qid, statics, dyn, nactive, blocks, t, s)
                           : step_s<F64, LBM_SRT>(qid, statics, dyn, nactive, blocks, t, s);
  if (storage == LBM_STORE_DF64_DEV)
    return coll == LBM_TRT ? step_s<DF64Dev, LBM_TRT>(qid, statics, dyn, nactive, blocks, t, s)
                           : step_s<DF64Dev, LBM_SRT>(qid, statics, dyn, nactive, blocks, t, s);
  if (storage == LBM_STORE_F32_DEV)
    return coll == LBM_TRT ? step_s<F32Dev, LBM_TRT>(qid, statics, dyn, nactive, blocks, t, s)
                           : step_s<F32Dev, LBM_SRT>(qid, statics, dyn, nactive, blocks, t, s);
  return cudaErrorInvalidValue;
}

// Reductions of the `nmem` members (in launch order) of one velocity set: partial sums from
// block part_base on, one row of kRedMaxK doubles per member (by static index) in `out`.
cudaError_t batch_reduce_launch(int storage, int qid, int K, const void* statics, const ReduceArgs* args,
                                const BatchDyn* dyn, int nmem, long long blocks, double* partial, long long part_base,
                                double* out, cudaStream_t s) {
  if (blocks <= 0 || nmem <= 0) return cudaSuccess;
  if (storage == LBM_STORE_F64) return reduce_s<F64>(qid, K, statics, args, dyn, nmem, blocks, partial, part_base, out, s);
  if (storage == LBM_STORE_DF64_DEV)
    return reduce_s<DF64Dev>(qid, K, statics, args, dyn, nmem, blocks, partial, part_base, out, s);
  if (storage == LBM_STORE_F32_DEV)
    return reduce_s<F32Dev>(qid, K, statics, args, dyn, nmem, blocks, partial, part_base, out, s);
  return cudaErrorInvalidValue;
}

size_t batch_static_size(int storage) {
  if (storage == LBM_STORE_F64) return sizeof(BatchStatic<double>);
  if (storage == LBM_STORE_DF64_DEV) return sizeof(BatchStatic<dd>);
  return sizeof(BatchStatic<float>);
}

}  // namespace lbm
