// Diagnostics on the device: the quadrature-weighted sums of check_conservation
// (src/dg/utils.jl:1-12) and the error norms of calculate_error (src/dg/postprocess.jl:1-46).
// Two passes with a fixed grid and fixed reduction trees, so a result does not depend on
// scheduling: each block reduces a fixed stride of nodes, one block reduces the blocks.
#include <cuda_runtime.h>

#include "p2de_diag.h"

namespace p2de {

namespace {

constexpr int kThreads = 256;

// per thread: for each component c, the values v[q * 4 + c], q < NQ; sums or maxima
template <int NQ>
__device__ void block_reduce(double (&v)[NQ * 4], const bool (&is_max)[NQ], double* out) {
  __shared__ double sh[kThreads];
  for (int q = 0; q < NQ; ++q)
    for (int c = 0; c < 4; ++c) {
      sh[threadIdx.x] = v[q * 4 + c];
      __syncthreads();
      for (int o = kThreads / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
          double a = sh[threadIdx.x], b = sh[threadIdx.x + o];
          sh[threadIdx.x] = is_max[q] ? fmax(a, b) : a + b;
        }
        __syncthreads();
      }
      if (threadIdx.x == 0) out[q * 4 + c] = sh[0];
      __syncthreads();
    }
}

// pass 1 of check_conservation: sum of J_k wq_i U[i,k,c] over this block's nodes
__global__ void k_wsum(const double* Uq, const double* geom, const double* wq, int Nq, long long nodes,
                       double* partial) {
  double v[4] = {0, 0, 0, 0};
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x; g < nodes; g += stride) {
    const long long k = g / Nq;
    const int i = (int)(g % Nq);
    const double w = geom[5 * k] * wq[i];
#pragma unroll
    for (int c = 0; c < 4; ++c) v[c] = fma(w, Uq[4 * g + c], v[c]);
  }
  const bool is_max[1] = {false};
  block_reduce<1>(v, is_max, partial + 4 * blockIdx.x);
}

// pass 1 of calculate_error: per component L1/L2 error, Linf error, L1/L2 exact, Linf exact
__global__ void k_err(const double* Uq, const double* Ue, const double* geom, const double* wq, int Nq,
                      long long nodes, double* partial) {
  double v[24];
#pragma unroll
  for (int j = 0; j < 24; ++j) v[j] = 0.0;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x; g < nodes; g += stride) {
    const long long k = g / Nq;
    const int i = (int)(g % Nq);
    const double w = wq[i] * geom[5 * k];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const double ex = Ue[4 * g + c], d = fabs(ex - Uq[4 * g + c]), ax = fabs(ex);
      v[0 * 4 + c] = fma(w, d, v[0 * 4 + c]);
      v[1 * 4 + c] = fma(w, d * d, v[1 * 4 + c]);
      v[2 * 4 + c] = fmax(v[2 * 4 + c], d);
      v[3 * 4 + c] = fma(w, ax, v[3 * 4 + c]);
      v[4 * 4 + c] = fma(w, ax * ax, v[4 * 4 + c]);
      v[5 * 4 + c] = fmax(v[5 * 4 + c], ax);
    }
  }
  const bool is_max[6] = {false, false, true, false, false, true};
  block_reduce<6>(v, is_max, partial + 24 * blockIdx.x);
}

// pass 2: one block reduces nblocks partial vectors of width W in block order
template <int NQ>
__global__ void k_final(const double* partial, int nblocks, const bool* is_max_q, double* out) {
  double v[NQ * 4];
  bool is_max[NQ];
  for (int q = 0; q < NQ; ++q) is_max[q] = is_max_q[q];
  for (int j = 0; j < NQ * 4; ++j) v[j] = 0.0;
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x)
    for (int q = 0; q < NQ; ++q)
      for (int c = 0; c < 4; ++c) {
        const double x = partial[(long long)b * NQ * 4 + q * 4 + c];
        v[q * 4 + c] = is_max[q] ? fmax(v[q * 4 + c], x) : v[q * 4 + c] + x;
      }
  block_reduce<NQ>(v, is_max, out);
}

__constant__ bool c_sum1[1] = {false};
__constant__ bool c_err6[6] = {false, false, true, false, false, true};

}  // namespace

int diag_blocks(int sms) { return 2 * sms; }

cudaError_t launch_weighted_sum(const double* Uq, const double* geom, const double* wq, int Nq, long long nodes,
                                int nblocks, double* partial, double* out4, cudaStream_t st) {
  k_wsum<<<nblocks, kThreads, 0, st>>>(Uq, geom, wq, Nq, nodes, partial);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const bool* flags = nullptr;
  e = cudaGetSymbolAddress((void**)&flags, c_sum1);
  if (e != cudaSuccess) return e;
  k_final<1><<<1, kThreads, 0, st>>>(partial, nblocks, flags, out4);
  return cudaGetLastError();
}

cudaError_t launch_error_norms(const double* Uq, const double* Ue, const double* geom, const double* wq, int Nq,
                               long long nodes, int nblocks, double* partial, double* out24, cudaStream_t st) {
  k_err<<<nblocks, kThreads, 0, st>>>(Uq, Ue, geom, wq, Nq, nodes, partial);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const bool* flags = nullptr;
  e = cudaGetSymbolAddress((void**)&flags, c_err6);
  if (e != cudaSuccess) return e;
  k_final<6><<<1, kThreads, 0, st>>>(partial, nblocks, flags, out24);
  return cudaGetLastError();
}

}  // namespace p2de
