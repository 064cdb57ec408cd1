// Batched stage kernel A with FP32 flux differencing (mixed precision).
#include "p2de_batch_kernels.cuh"
#include "p2de_batch_launch.h"

namespace p2de {

cudaError_t batch_prepare_f64();
cudaError_t batch_occupancy_f64(size_t smem_a, size_t smem_b, int* bpa, int* bpb);
cudaError_t launch_batch_a_f64(int grid, size_t smem, const StageArgs* solves, const BatchTask* tasks,
                               const int* ntasks, unsigned* counter, int nstage, cudaStream_t st);

cudaError_t batch_prepare(bool mixed) {
  cudaError_t e = batch_prepare_f64();
  if (e != cudaSuccess || !mixed) return e;
  return cudaFuncSetAttribute(k_batch_a<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kBatchSmemAMax);
}

cudaError_t batch_occupancy(bool mixed, size_t smem_a, size_t smem_b, int* bpa, int* bpb) {
  cudaError_t e = batch_occupancy_f64(smem_a, smem_b, bpa, bpb);
  if (e != cudaSuccess || !mixed) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(bpa, k_batch_a<float>, kBatchThreads, smem_a);
}

cudaError_t launch_batch_a(bool mixed, int grid, size_t smem, const StageArgs* solves, const BatchTask* tasks,
                           const int* ntasks, unsigned* counter, int nstage, cudaStream_t st) {
  if (!mixed) return launch_batch_a_f64(grid, smem, solves, tasks, ntasks, counter, nstage, st);
  k_batch_a<float><<<grid, kBatchThreads, smem, st>>>(solves, tasks, ntasks, counter, nstage);
  return cudaGetLastError();
}

}  // namespace p2de
