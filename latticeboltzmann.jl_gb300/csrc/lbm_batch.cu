// lbm_batch.cu -- dispatch of the batched kernels (lbm_batch.cuh) to the per-velocity-set
// instantiations of lbm_batch_q*.cu.
#include "lbm_resident.cuh"

namespace lbm {

cudaError_t batch_launch_q4(int, int, const void*, const BatchDyn*, int, long long, long long, cudaStream_t);
cudaError_t batch_reduce_q4(int, int, const void*, const ReduceArgs*, const BatchDyn*, int, long long, double*, long long,
                            double*, cudaStream_t);
cudaError_t batch_launch_q5(int, int, const void*, const BatchDyn*, int, long long, long long, cudaStream_t);
cudaError_t batch_reduce_q5(int, int, const void*, const ReduceArgs*, const BatchDyn*, int, long long, double*, long long,
                            double*, cudaStream_t);
cudaError_t batch_launch_q9(int, int, const void*, const BatchDyn*, int, long long, long long, cudaStream_t);
cudaError_t batch_reduce_q9(int, int, const void*, const ReduceArgs*, const BatchDyn*, int, long long, double*, long long,
                            double*, cudaStream_t);
cudaError_t batch_launch_q13(int, int, const void*, const BatchDyn*, int, long long, long long, cudaStream_t);
cudaError_t batch_reduce_q13(int, int, const void*, const ReduceArgs*, const BatchDyn*, int, long long, double*, long long,
                            double*, cudaStream_t);
cudaError_t batch_launch_q17(int, int, const void*, const BatchDyn*, int, long long, long long, cudaStream_t);
cudaError_t batch_reduce_q17(int, int, const void*, const ReduceArgs*, const BatchDyn*, int, long long, double*, long long,
                            double*, cudaStream_t);
cudaError_t batch_launch_q21(int, int, const void*, const BatchDyn*, int, long long, long long, cudaStream_t);
cudaError_t batch_reduce_q21(int, int, const void*, const ReduceArgs*, const BatchDyn*, int, long long, double*, long long,
                            double*, cudaStream_t);
cudaError_t batch_launch_q37(int, int, const void*, const BatchDyn*, int, long long, long long, cudaStream_t);
cudaError_t batch_reduce_q37(int, int, const void*, const ReduceArgs*, const BatchDyn*, int, long long, double*, long long,
                            double*, cudaStream_t);

cudaError_t resident_launch_q4(int, int, const void*, const ResidentDyn*, int, int, int, int, int, size_t, cudaStream_t);
cudaError_t resident_launch_q5(int, int, const void*, const ResidentDyn*, int, int, int, int, int, size_t, cudaStream_t);
cudaError_t resident_launch_q9(int, int, const void*, const ResidentDyn*, int, int, int, int, int, size_t, cudaStream_t);
cudaError_t resident_launch_q13(int, int, const void*, const ResidentDyn*, int, int, int, int, int, size_t, cudaStream_t);
cudaError_t resident_launch_q17(int, int, const void*, const ResidentDyn*, int, int, int, int, int, size_t, cudaStream_t);
cudaError_t resident_launch_q21(int, int, const void*, const ResidentDyn*, int, int, int, int, int, size_t, cudaStream_t);
cudaError_t resident_launch_q37(int, int, const void*, const ResidentDyn*, int, int, int, int, int, size_t, cudaStream_t);

namespace {
using ResidentFn = cudaError_t (*)(int, int, const void*, const ResidentDyn*, int, int, int, int, int, size_t, cudaStream_t);
const ResidentFn kResident[7] = {resident_launch_q4, resident_launch_q5, resident_launch_q9, resident_launch_q13,
                                 resident_launch_q17, resident_launch_q21, resident_launch_q37};
using StepFn = cudaError_t (*)(int, int, const void*, const BatchDyn*, int, long long, long long, cudaStream_t);
using ReduceFn = cudaError_t (*)(int, int, const void*, const ReduceArgs*, const BatchDyn*, int, long long, double*,
                                 long long, double*, cudaStream_t);
const StepFn kStep[7] = {batch_launch_q4, batch_launch_q5, batch_launch_q9, batch_launch_q13,
                         batch_launch_q17, batch_launch_q21, batch_launch_q37};
const ReduceFn kReduce[7] = {batch_reduce_q4, batch_reduce_q5, batch_reduce_q9, batch_reduce_q13,
                             batch_reduce_q17, batch_reduce_q21, batch_reduce_q37};
}  // namespace

// One global step t for the first `nactive` members (in launch order) of one velocity set.
cudaError_t batch_launch(int storage, int coll, int qid, const void* statics, const BatchDyn* dyn, int nactive,
                         long long blocks, long long t, cudaStream_t s) {
  if (qid < 0 || qid > 6) return cudaErrorInvalidValue;
  return kStep[qid](storage, coll, statics, dyn, nactive, blocks, t, s);
}

// Reductions of the `nmem` members (in launch order) of one velocity set.
cudaError_t batch_reduce_launch(int storage, int qid, int K, const void* statics, const ReduceArgs* args,
                                const BatchDyn* dyn, int nmem, long long blocks, double* partial, long long part_base,
                                double* out, cudaStream_t s) {
  if (qid < 0 || qid > 6) return cudaErrorInvalidValue;
  return kReduce[qid](storage, K, statics, args, dyn, nmem, blocks, partial, part_base, out, s);
}

// All steps of one call for `nmem` block-resident members of one velocity set (lbm_resident.cuh).
cudaError_t resident_launch(int storage, int coll, int qid, const void* statics, const ResidentDyn* dyn, int nmem,
                            int csize, int stride, int threads, int parts, size_t smem_min, cudaStream_t s) {
  if (qid < 0 || qid > 6) return cudaErrorInvalidValue;
  return kResident[qid](storage, coll, statics, dyn, nmem, csize, stride, threads, parts, smem_min, s);
}

size_t batch_static_size(int storage) {
  if (storage == LBM_STORE_F64) return sizeof(BatchStatic<double>);
  if (storage == LBM_STORE_DF64_DEV) return sizeof(BatchStatic<dd>);
  return sizeof(BatchStatic<float>);
}

}  // namespace lbm
