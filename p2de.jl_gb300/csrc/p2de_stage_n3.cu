// Stage kernels for N1D = 3 (polynomial degree 2).
#include "p2de_stage_impl.cuh"

namespace p2de {
template cudaError_t stage_prepare<3>(StageGeometry*);
template cudaError_t launch_stage_a<3>(const StageArgs&, bool, cudaStream_t);
template cudaError_t launch_stage_b<3>(const StageArgs&, cudaStream_t);
template cudaError_t launch_gauss_proj<3>(const StageArgs&, cudaStream_t);
template cudaError_t launch_es_interface<3>(const StageArgs&, cudaStream_t);
}  // namespace p2de
