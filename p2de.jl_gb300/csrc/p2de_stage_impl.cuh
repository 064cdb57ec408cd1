// Generic definitions of the launchers; each p2de_stage_n<N1D>.cu instantiates one N1D.
#pragma once

#include "p2de_launch.h"
#include "p2de_stage.cuh"

namespace p2de {

template <int N1D>
cudaError_t stage_prepare(StageGeometry* geo) {
  using C = Cfg<N1D>;
  cudaError_t e;
  e = cudaFuncSetAttribute(k_stage_a<N1D, double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)C::SMEM_A);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_stage_a<N1D, float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)C::SMEM_A);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_stage_b<N1D>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)C::SMEM_B);
  if (e != cudaSuccess) return e;
  geo->elems_per_block = C::E;
  geo->threads = C::THREADS;
  geo->smem_a = C::SMEM_A;
  geo->smem_b = C::SMEM_B;
  geo->fbar_per_elem = C::FBAR;
  geo->nsf = C::NSF;
  return cudaSuccess;
}

template <int N1D>
cudaError_t launch_stage_a(const StageArgs& a, bool mixed, cudaStream_t st) {
  using C = Cfg<N1D>;
  int grid = (a.K + C::E - 1) / C::E;
  if (mixed)
    k_stage_a<N1D, float><<<grid, C::THREADS, C::SMEM_A, st>>>(a);
  else
    k_stage_a<N1D, double><<<grid, C::THREADS, C::SMEM_A, st>>>(a);
  return cudaGetLastError();
}

template <int N1D>
cudaError_t launch_stage_b(const StageArgs& a, cudaStream_t st) {
  using C = Cfg<N1D>;
  int grid = (a.K + C::E - 1) / C::E;
  k_stage_b<N1D><<<grid, C::THREADS, C::SMEM_B, st>>>(a);
  return cudaGetLastError();
}

}  // namespace p2de
