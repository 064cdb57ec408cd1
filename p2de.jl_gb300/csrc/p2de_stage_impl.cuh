// Generic definitions of the launchers; each p2de_stage_n<N1D>.cu instantiates one N1D.
#pragma once

#include "p2de_launch.h"
#include "p2de_stage.cuh"

namespace p2de {

template <int N1D>
cudaError_t stage_prepare(StageGeometry* geo) {
  using C = Cfg<N1D>;
  cudaError_t e;
  e = cudaFuncSetAttribute(k_stage_a<N1D, double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)C::smem_a(C::E_MAX));
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_stage_a<N1D, float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)C::smem_a(C::E_MAX));
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_stage_b<N1D>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)C::smem_b(C::E_MAX));
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_stage_a<N1D, double, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)C::smem_g(C::E_MAX_G));
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_stage_a<N1D, double, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)C::smem_x(C::E_MAX));
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_stage_a<N1D, float, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)C::smem_x(C::E_MAX));
  if (e != cudaSuccess) return e;
  geo->elems_per_block = C::E;
  geo->elems_per_block_max = C::E_MAX;
  geo->elems_per_block_gauss = C::E_G;
  geo->elems_per_block_max_gauss = C::E_MAX_G;
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
  if (a.flags & F_GAUSS) {
    if (mixed || a.epb < 1 || a.epb > C::E_MAX_G) return cudaErrorInvalidValue;
    int grid = (a.K + a.epb - 1) / a.epb;
    k_stage_a<N1D, double, true, true><<<grid, C::THREADS, C::smem_g(a.epb), st>>>(a);
    return cudaGetLastError();
  }
  if (a.epb < 1 || a.epb > C::E_MAX) return cudaErrorInvalidValue;
  const int th = a.threads > 0 ? a.threads : C::THREADS;
  if (th % 32 != 0 || th > C::THREADS) return cudaErrorInvalidValue;
  int grid = (a.K + a.epb - 1) / a.epb;
  const bool ext = a.flags & kExtFlags;
  if (mixed && ext)
    k_stage_a<N1D, float, false, true><<<grid, th, C::smem_x(a.epb), st>>>(a);
  else if (mixed)
    k_stage_a<N1D, float><<<grid, th, C::smem_a(a.epb), st>>>(a);
  else if (ext)
    k_stage_a<N1D, double, false, true><<<grid, th, C::smem_x(a.epb), st>>>(a);
  else
    k_stage_a<N1D, double><<<grid, th, C::smem_a(a.epb), st>>>(a);
  return cudaGetLastError();
}

template <int N1D>
cudaError_t launch_gauss_proj(const StageArgs& a, cudaStream_t st) {
  using C = Cfg<N1D>;
  if (a.epb < 1 || a.epb > C::E_MAX_G) return cudaErrorInvalidValue;
  int grid = (a.K + a.epb - 1) / a.epb;
  k_gauss_proj<N1D><<<grid, C::THREADS, C::smem_p(a.epb), st>>>(a);
  return cudaGetLastError();
}

template <int N1D>
cudaError_t launch_es_interface(const StageArgs& a, cudaStream_t st) {
  const long long items = (long long)a.K * Cfg<N1D>::Nfp;
  k_es_interface<N1D><<<(int)((items + 255) / 256), 256, 0, st>>>(a);
  return cudaGetLastError();
}

// Kernel B runs C::E elements per block whatever kernel A's tuned value is: its work per
// element is fixed and it is fastest at the default (at a quarter of that it ran 45% slower,
// which an autotuner timing kernel A alone would not see); its results do not depend on it.
template <int N1D>
cudaError_t launch_stage_b(const StageArgs& a, cudaStream_t st) {
  using C = Cfg<N1D>;
  StageArgs b = a;
  b.epb = C::E;
  int grid = (b.K + b.epb - 1) / b.epb;
  k_stage_b<N1D><<<grid, C::THREADS, C::smem_b(b.epb), st>>>(b);
  return cudaGetLastError();
}

}  // namespace p2de
