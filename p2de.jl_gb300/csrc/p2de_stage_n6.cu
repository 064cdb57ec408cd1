// Stage kernels for N1D = 6 (polynomial degree 5).
#include "p2de_stage_impl.cuh"

namespace p2de {
template cudaError_t stage_prepare<6>(StageGeometry*);
template cudaError_t launch_stage_a<6>(const StageArgs&, bool, cudaStream_t);
template cudaError_t launch_stage_b<6>(const StageArgs&, cudaStream_t);
template cudaError_t launch_gauss_proj<6>(const StageArgs&, cudaStream_t);
template cudaError_t launch_es_interface<6>(const StageArgs&, cudaStream_t);
}  // namespace p2de
