// Batched stage kernel A with FP32 flux differencing (mixed precision).
#include "p2de_batch_kernels.cuh"
#include "p2de_batch_launch.h"

namespace p2de {

cudaError_t batch_prepare_f64();
cudaError_t batch_occupancy_f64(bool ext, size_t smem_a, size_t smem_b, int* bpa, int* bpb);
cudaError_t launch_batch_a_f64(bool ext, int mode, int grid, size_t smem, const StageArgs* solves,
                               const BatchTask* tasks, const int* ntasks, unsigned* counter, int nstage,
                               cudaStream_t st);

cudaError_t batch_prepare(bool mixed) {
  cudaError_t e = batch_prepare_f64();
  if (e != cudaSuccess || !mixed) return e;
  e = cudaFuncSetAttribute(k_batch_a<float, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kBatchSmemAMax);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_batch_a<float, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kBatchSmemXMax);
}

cudaError_t batch_occupancy(bool mixed, bool ext, size_t smem_a, size_t smem_b, int* bpa, int* bpb) {
  cudaError_t e = batch_occupancy_f64(ext, smem_a, smem_b, bpa, bpb);
  if (e != cudaSuccess || !mixed) return e;
  return ext ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(bpa, k_batch_a<float, true>, kBatchThreads, smem_a)
             : cudaOccupancyMaxActiveBlocksPerMultiprocessor(bpa, k_batch_a<float, false>, kBatchThreads, smem_a);
}

cudaError_t launch_batch_a(bool mixed, bool ext, int mode, int grid, size_t smem, const StageArgs* solves,
                           const BatchTask* tasks, const int* ntasks, unsigned* counter, int nstage, cudaStream_t st) {
  if (!mixed) return launch_batch_a_f64(ext, mode, grid, smem, solves, tasks, ntasks, counter, nstage, st);
  if (ext)
    k_batch_a<float, true><<<grid, kBatchThreads, smem, st>>>(solves, tasks, ntasks, counter, nstage, mode);
  else
    k_batch_a<float, false><<<grid, kBatchThreads, smem, st>>>(solves, tasks, ntasks, counter, nstage, mode);
  return cudaGetLastError();
}

}  // namespace p2de
