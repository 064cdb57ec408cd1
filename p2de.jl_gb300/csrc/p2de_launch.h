// Per-N1D launchers of the stage kernels (instantiated in p2de_stage_n<N1D>.cu).
#pragma once

#include <cuda_runtime.h>

#include "p2de_args.h"

namespace p2de {

struct StageGeometry {
  int elems_per_block;      // default
  int elems_per_block_max;  // largest allowed (shared-memory limit)
  int threads;
  size_t smem_a;
  size_t smem_b;
  int fbar_per_elem;  // doubles of subcell flux data per element
  int nsf;            // subcell faces per direction (Nq + N1D)
  int elems_per_block_gauss;      // the same two for GaussCollocation's kernel A
  int elems_per_block_max_gauss;
};

template <int N1D>
cudaError_t stage_prepare(StageGeometry* geo);
template <int N1D>
cudaError_t launch_stage_a(const StageArgs& a, bool mixed, cudaStream_t st);
template <int N1D>
cudaError_t launch_stage_b(const StageArgs& a, cudaStream_t st);
template <int N1D>
cudaError_t launch_gauss_proj(const StageArgs& a, cudaStream_t st);
template <int N1D>
cudaError_t launch_es_interface(const StageArgs& a, cudaStream_t st);

// Per-element geometry factors (geom_factor) for K elements: out has 16 doubles per element.
cudaError_t launch_geom_table(const double* geom, int K, double* out, cudaStream_t st);

}  // namespace p2de
