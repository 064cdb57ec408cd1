// Launchers of the batched stage kernels (p2de_batch_f64.cu, p2de_batch_f32.cu).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "p2de_args.h"

namespace p2de {

struct BatchTask;

// Sets the kernels' largest shared-memory limits.
cudaError_t batch_prepare(bool mixed);
// Resident blocks per SM of the stage kernels at the given dynamic shared memory (kernel A
// in its plain or EXT instantiation).
cudaError_t batch_occupancy(bool mixed, bool ext, size_t smem_a, size_t smem_b, int* blocks_per_sm_a,
                            int* blocks_per_sm_b);
// Batched kernel A over a task list: plain or EXT instantiation, full or low-only pass (mode).
cudaError_t launch_batch_a(bool mixed, bool ext, int mode, int grid, size_t smem, const StageArgs* solves,
                           const BatchTask* tasks, const int* ntasks, unsigned* counter, int nstage, cudaStream_t st);
// initialize_s_modified! of the members with a relaxed min-entropy bound (one block per slot).
cudaError_t launch_batch_phi_min(const StageArgs* solves, const uint8_t* active, int nslots, cudaStream_t st);
cudaError_t launch_batch_b(int grid, size_t smem, const StageArgs* solves, const BatchTask* tasks, const int* ntasks,
                           unsigned* counter, int nstage, cudaStream_t st);
cudaError_t launch_batch_begin(const StageArgs* solves, const uint8_t* active, int nslots, unsigned* counters,
                               cudaStream_t st);
int batch_elems_per_block(int n1d);      // default
int batch_elems_per_block_max(int n1d);  // shared-memory limit
size_t batch_smem_a(int n1d, int epb, bool ext = false);
size_t batch_smem_b(int n1d, int epb);

}  // namespace p2de
