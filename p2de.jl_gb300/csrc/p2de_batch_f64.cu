// Batched stage kernels, FP64 flux differencing; kernel B and the step begin.
#define P2DE_BATCH_COMMON_KERNELS
#include "p2de_batch_kernels.cuh"
#include "p2de_batch_launch.h"

namespace p2de {

cudaError_t batch_prepare_f64() {
  cudaError_t e = cudaFuncSetAttribute(k_batch_a<double, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)kBatchSmemAMax);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_batch_a<double, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kBatchSmemXMax);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_batch_b, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kBatchSmemBMax);
}

cudaError_t batch_occupancy_f64(bool ext, size_t smem_a, size_t smem_b, int* bpa, int* bpb) {
  cudaError_t e = ext ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(bpa, k_batch_a<double, true>, kBatchThreads, smem_a)
                      : cudaOccupancyMaxActiveBlocksPerMultiprocessor(bpa, k_batch_a<double, false>, kBatchThreads, smem_a);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(bpb, k_batch_b, kBatchThreads, smem_b);
}

cudaError_t launch_batch_a_f64(bool ext, int mode, int grid, size_t smem, const StageArgs* solves,
                               const BatchTask* tasks, const int* ntasks, unsigned* counter, int nstage,
                               cudaStream_t st) {
  if (ext)
    k_batch_a<double, true><<<grid, kBatchThreads, smem, st>>>(solves, tasks, ntasks, counter, nstage, mode);
  else
    k_batch_a<double, false><<<grid, kBatchThreads, smem, st>>>(solves, tasks, ntasks, counter, nstage, mode);
  return cudaGetLastError();
}

cudaError_t launch_batch_phi_min(const StageArgs* solves, const uint8_t* active, int nslots, cudaStream_t st) {
  k_batch_phi_min<<<nslots > 0 ? nslots : 1, 1024, 0, st>>>(solves, active, nslots);
  return cudaGetLastError();
}

cudaError_t launch_batch_b(int grid, size_t smem, const StageArgs* solves, const BatchTask* tasks, const int* ntasks,
                           unsigned* counter, int nstage, cudaStream_t st) {
  k_batch_b<<<grid, kBatchThreads, smem, st>>>(solves, tasks, ntasks, counter, nstage);
  return cudaGetLastError();
}

cudaError_t launch_batch_begin(const StageArgs* solves, const uint8_t* active, int nslots, unsigned* counters,
                               cudaStream_t st) {
  int grid = (nslots + 127) / 128;
  k_batch_begin<<<grid > 0 ? grid : 1, 128, 0, st>>>(solves, active, nslots, counters);
  return cudaGetLastError();
}

int batch_elems_per_block(int n1d) {
  switch (n1d) {
    case 2: return Cfg<2>::E;
    case 3: return Cfg<3>::E;
    case 4: return Cfg<4>::E;
    case 5: return Cfg<5>::E;
    case 6: return Cfg<6>::E;
  }
  return 0;
}

int batch_elems_per_block_max(int n1d) {
  switch (n1d) {
    case 2: return Cfg<2>::E_MAX;
    case 3: return Cfg<3>::E_MAX;
    case 4: return Cfg<4>::E_MAX;
    case 5: return Cfg<5>::E_MAX;
    case 6: return Cfg<6>::E_MAX;
  }
  return 0;
}

size_t batch_smem_a(int n1d, int epb, bool ext) {
  switch (n1d) {
    case 2: return ext ? Cfg<2>::smem_x(epb) : Cfg<2>::smem_a(epb);
    case 3: return ext ? Cfg<3>::smem_x(epb) : Cfg<3>::smem_a(epb);
    case 4: return ext ? Cfg<4>::smem_x(epb) : Cfg<4>::smem_a(epb);
    case 5: return ext ? Cfg<5>::smem_x(epb) : Cfg<5>::smem_a(epb);
    case 6: return ext ? Cfg<6>::smem_x(epb) : Cfg<6>::smem_a(epb);
  }
  return 0;
}

size_t batch_smem_b(int n1d, int epb) {
  switch (n1d) {
    case 2: return Cfg<2>::smem_b(epb);
    case 3: return Cfg<3>::smem_b(epb);
    case 4: return Cfg<4>::smem_b(epb);
    case 5: return Cfg<5>::smem_b(epb);
    case 6: return Cfg<6>::smem_b(epb);
  }
  return 0;
}

}  // namespace p2de
