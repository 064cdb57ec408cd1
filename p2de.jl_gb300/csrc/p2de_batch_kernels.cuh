// Batched stage kernels: one persistent launch per RK stage advances every active
// solve of a batch, whatever their mesh sizes and polynomial degrees. Blocks take
// tasks (solve, first element, N+1) from a device work list through an atomic
// counter, copy the solve's descriptor into shared memory and run the same stage
// bodies as the one-solve kernels, so a solve's result in a batch is bitwise the
// result it has alone.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "p2de_args.h"
#include "p2de_stage.cuh"

namespace p2de {

struct BatchTask {
  int32_t solve;  // slot of the solve descriptor
  int32_t k0;     // first element of the task
  int32_t n1d;    // N + 1 of the solve
  int32_t epb;    // elements in this task (<= the degree's elements per block)
  int32_t layout; // thread layout of the pair phases for this degree (StageArgs::layout)
};

constexpr int kBatchThreads = 128;

__host__ __device__ constexpr size_t smax(size_t a, size_t b) { return a > b ? a : b; }
// largest dynamic shared memory the batched kernels may be launched with: the largest
// over N1D = 2..6 at each degree's maximum elements per block
constexpr size_t kBatchSmemAMax =
    smax(smax(smax(Cfg<2>::smem_a(Cfg<2>::E_MAX), Cfg<3>::smem_a(Cfg<3>::E_MAX)),
              smax(Cfg<4>::smem_a(Cfg<4>::E_MAX), Cfg<5>::smem_a(Cfg<5>::E_MAX))),
         Cfg<6>::smem_a(Cfg<6>::E_MAX));
constexpr size_t kBatchSmemXMax =
    smax(smax(smax(Cfg<2>::smem_x(Cfg<2>::E_MAX), Cfg<3>::smem_x(Cfg<3>::E_MAX)),
              smax(Cfg<4>::smem_x(Cfg<4>::E_MAX), Cfg<5>::smem_x(Cfg<5>::E_MAX))),
         Cfg<6>::smem_x(Cfg<6>::E_MAX));
constexpr size_t kBatchSmemBMax =
    smax(smax(smax(Cfg<2>::smem_b(Cfg<2>::E_MAX), Cfg<3>::smem_b(Cfg<3>::E_MAX)),
              smax(Cfg<4>::smem_b(Cfg<4>::E_MAX), Cfg<5>::smem_b(Cfg<5>::E_MAX))),
         Cfg<6>::smem_b(Cfg<6>::E_MAX));

// passes of batched kernel A: the full stage body, or (TVD bounds) the pass that stops
// after the low-order RHS and stores the low-order densities (the one-solve path's first
// kernel A launch of such a stage)
enum : int { BATCH_A_FULL = 0, BATCH_A_LOW_ONLY = 1 };
// task counters per step: kBatchCountersPerStage per stage (kernel A passes and kernel B)
constexpr int kBatchCountersPerStage = 5;
constexpr int kBatchCounters = 3 * kBatchCountersPerStage;

// Fetches the next task; returns false when the list is exhausted. The solve's
// descriptor lands in `sa` with the stage's flags: F_UPDATE always, F_CFL at stage 1, and
// for the low-only pass F_LOW_ONLY without F_CFL.
__device__ __forceinline__ bool batch_next(const StageArgs* solves, const BatchTask* tasks, const int* ntasks,
                                           unsigned* counter, int nstage, StageArgs& sa, BatchTask& tk, int& s_task,
                                           int mode = BATCH_A_FULL) {
  __syncthreads();  // the previous task's shared data is no longer read
  if (threadIdx.x == 0) s_task = (int)atomicAdd(counter, 1u);
  __syncthreads();
  const int t = s_task;
  if (t >= *ntasks) return false;
  tk = tasks[t];
  const int* src = reinterpret_cast<const int*>(solves + tk.solve);
  int* dst = reinterpret_cast<int*>(&sa);
  for (int i = threadIdx.x; i < (int)(sizeof(StageArgs) / sizeof(int)); i += blockDim.x) dst[i] = src[i];
  __syncthreads();
  if (threadIdx.x == 0) {
    sa.nstage = nstage;
    sa.epb = tk.epb;
    sa.layout = tk.layout;
    int f = sa.flags | F_UPDATE;
    if (nstage == 1 && (f & F_DO_LOW)) f |= F_CFL;
    if (mode == BATCH_A_LOW_ONLY) f = (f | F_LOW_ONLY) & ~(F_CFL | F_WRITE_DEBUG);
    sa.flags = f;
  }
  __syncthreads();
  return true;
}

// EXT: the instantiation of the stage body that compiles the rarely used modes (Zhang-Shu,
// min-entropy and relaxed bounds, the projected low-order flux), for the members that use
// them; the others run the plain one, each member the same instantiation as alone.
template <typename TH, bool EXT>
__global__ void __launch_bounds__(kBatchThreads) k_batch_a(const StageArgs* solves, const BatchTask* tasks,
                                                           const int* ntasks, unsigned* counter, int nstage, int mode) {
  extern __shared__ __align__(16) double sm[];
  __shared__ StageArgs sa;
  __shared__ int s_task;
  BatchTask tk;
  while (batch_next(solves, tasks, ntasks, counter, nstage, sa, tk, s_task, mode)) {
    switch (tk.n1d) {
      case 2: stage_a_body<2, TH, false, EXT>(sa, tk.k0, sm); break;
      case 3: stage_a_body<3, TH, false, EXT>(sa, tk.k0, sm); break;
      case 4: stage_a_body<4, TH, false, EXT>(sa, tk.k0, sm); break;
      case 5: stage_a_body<5, TH, false, EXT>(sa, tk.k0, sm); break;
      case 6: stage_a_body<6, TH, false, EXT>(sa, tk.k0, sm); break;
    }
  }
}

// Kernel B and the step begin are defined in one translation unit only.
#ifdef P2DE_BATCH_COMMON_KERNELS
__global__ void __launch_bounds__(kBatchThreads) k_batch_b(const StageArgs* solves, const BatchTask* tasks,
                                                           const int* ntasks, unsigned* counter, int nstage) {
  extern __shared__ __align__(16) double sm[];
  __shared__ StageArgs sa;
  __shared__ int s_task;
  BatchTask tk;
  while (batch_next(solves, tasks, ntasks, counter, nstage, sa, tk, s_task)) {
    switch (tk.n1d) {
      case 2: stage_b_body<2>(sa, tk.k0, sm); break;
      case 3: stage_b_body<3>(sa, tk.k0, sm); break;
      case 4: stage_b_body<4>(sa, tk.k0, sm); break;
      case 5: stage_b_body<5>(sa, tk.k0, sm); break;
      case 6: stage_b_body<6>(sa, tk.k0, sm); break;
    }
  }
}

// Step begin for every slot (SSPRK33.jl:126 per solve) and reset of the six task
// counters of the step. scal/dtmin/minrec/status are slot-indexed arrays.
__global__ void k_batch_begin(const StageArgs* solves, const uint8_t* active, int nslots, unsigned* counters) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s == 0)
    for (int i = 0; i < kBatchCounters; ++i) counters[i] = 0u;
  if (s >= nslots || !active[s]) return;
  const StageArgs& a = solves[s];
  double* scal = a.scal;
  double t = scal[S_T];
  if (!(t < a.T) || *a.status != 0) {
    scal[S_DONE] = 1.0;
    return;
  }
  scal[S_DONE] = 0.0;
  double dt = fmin(a.CFL * a.dt0, a.T - t);
  scal[S_DT_LIM] = dt;
  if (!(dt > 0.0)) {
    atomicOr(a.status, ST_BAD_DT);
    scal[S_DONE] = 1.0;
    return;
  }
  *a.dtmin_bits = (unsigned long long)__double_as_longlong(dt);
  for (int i = 0; i < 6; ++i) a.minrec[i] = 0x7ff0000000000000LL;
}

// initialize_s_modified! of every member with a relaxed min-entropy bound, at its t0,
// stage 1: one block of 1024 threads per slot, the one-solve kernel's body.
__global__ void __launch_bounds__(1024) k_batch_phi_min(const StageArgs* solves, const uint8_t* active, int nslots) {
  const int s = blockIdx.x;
  if (s >= nslots || !active[s]) return;
  const StageArgs& a = solves[s];
  if (!((a.flags & F_MIN_ENTROPY) && (a.flags & F_RELAXED))) return;
  const int n1d = a.ops->N1D;
  phi_min_body(a.Uq, (size_t)a.K * n1d * n1d, a.gamma, a.scal, a.t0, a.phimin);
}
#endif  // P2DE_BATCH_COMMON_KERNELS

}  // namespace p2de
