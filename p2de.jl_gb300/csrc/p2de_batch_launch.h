// Launchers of the batched stage kernels (p2de_batch_f64.cu, p2de_batch_f32.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "p2de_args.h"

namespace p2de {

struct BatchTask;

// Sets the kernels' shared-memory limits and returns resident blocks per SM of the
// stage kernels (the persistent grid is that times the SM count).
cudaError_t batch_prepare(bool mixed, int* blocks_per_sm_a, int* blocks_per_sm_b);
cudaError_t launch_batch_a(bool mixed, int grid, const StageArgs* solves, const BatchTask* tasks, const int* ntasks,
                           unsigned* counter, int nstage, cudaStream_t st);
cudaError_t launch_batch_b(int grid, const StageArgs* solves, const BatchTask* tasks, const int* ntasks,
                           unsigned* counter, int nstage, cudaStream_t st);
cudaError_t launch_batch_begin(const StageArgs* solves, const uint8_t* active, int nslots, unsigned* counters,
                               cudaStream_t st);
int batch_elems_per_block(int n1d);

}  // namespace p2de
