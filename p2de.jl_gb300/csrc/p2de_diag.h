// Launchers of the device diagnostics (p2de_diag.cu).
#pragma once

#include <cuda_runtime.h>

namespace p2de {

// blocks of the first pass (fixed per device, so results are reproducible)
int diag_blocks(int sms);

// out4[c] = sum over nodes of J_k wq_i Uq[i,k,c]; partial holds 4 * nblocks doubles
cudaError_t launch_weighted_sum(const double* Uq, const double* geom, const double* wq, int Nq, long long nodes,
                                int nblocks, double* partial, double* out4, cudaStream_t st);

// out24 = per component (4 each): sum wJ |e|, sum wJ e^2, max |e|, sum wJ |x|, sum wJ x^2,
// max |x|, with e = x - Uq and x the exact values; partial holds 24 * nblocks doubles
cudaError_t launch_error_norms(const double* Uq, const double* Ue, const double* geom, const double* wq, int Nq,
                               long long nodes, int nblocks, double* partial, double* out24, cudaStream_t st);

}  // namespace p2de
