// Stage kernels for N1D = 5 (polynomial degree 4).
#include "p2de_stage_impl.cuh"

namespace p2de {
template cudaError_t stage_prepare<5>(StageGeometry*);
template cudaError_t launch_stage_a<5>(const StageArgs&, bool, cudaStream_t);
template cudaError_t launch_stage_b<5>(const StageArgs&, cudaStream_t);
template cudaError_t launch_gauss_proj<5>(const StageArgs&, cudaStream_t);
template cudaError_t launch_es_interface<5>(const StageArgs&, cudaStream_t);
}  // namespace p2de
