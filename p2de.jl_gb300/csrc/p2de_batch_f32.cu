// Batched stage kernel A with FP32 flux differencing (mixed precision).
#include "p2de_batch_kernels.cuh"
#include "p2de_batch_launch.h"

namespace p2de {

cudaError_t batch_prepare_f64(int* bpa, int* bpb);
cudaError_t launch_batch_a_f64(int grid, const StageArgs* solves, const BatchTask* tasks, const int* ntasks,
                               unsigned* counter, int nstage, cudaStream_t st);

cudaError_t batch_prepare(bool mixed, int* bpa, int* bpb) {
  cudaError_t e = batch_prepare_f64(bpa, bpb);
  if (e != cudaSuccess || !mixed) return e;
  e = cudaFuncSetAttribute(k_batch_a<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kBatchSmemA);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(bpa, k_batch_a<float>, kBatchThreads, kBatchSmemA);
}

cudaError_t launch_batch_a(bool mixed, int grid, const StageArgs* solves, const BatchTask* tasks, const int* ntasks,
                           unsigned* counter, int nstage, cudaStream_t st) {
  if (!mixed) return launch_batch_a_f64(grid, solves, tasks, ntasks, counter, nstage, st);
  k_batch_a<float><<<grid, kBatchThreads, kBatchSmemA, st>>>(solves, tasks, ntasks, counter, nstage);
  return cudaGetLastError();
}

}  // namespace p2de
