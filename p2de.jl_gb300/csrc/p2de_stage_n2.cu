// Stage kernels for N1D = 2 (polynomial degree 1).
#include "p2de_stage_impl.cuh"

namespace p2de {
template cudaError_t stage_prepare<2>(StageGeometry*);
template cudaError_t launch_stage_a<2>(const StageArgs&, bool, cudaStream_t);
template cudaError_t launch_stage_b<2>(const StageArgs&, cudaStream_t);
template cudaError_t launch_gauss_proj<2>(const StageArgs&, cudaStream_t);
template cudaError_t launch_es_interface<2>(const StageArgs&, cudaStream_t);
}  // namespace p2de
