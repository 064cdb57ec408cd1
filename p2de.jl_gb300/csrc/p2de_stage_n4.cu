// Stage kernels for N1D = 4 (polynomial degree 3).
#include "p2de_stage_impl.cuh"

namespace p2de {
template cudaError_t stage_prepare<4>(StageGeometry*);
template cudaError_t launch_stage_a<4>(const StageArgs&, bool, cudaStream_t);
template cudaError_t launch_stage_b<4>(const StageArgs&, cudaStream_t);
template cudaError_t launch_gauss_proj<4>(const StageArgs&, cudaStream_t);
template cudaError_t launch_es_interface<4>(const StageArgs&, cudaStream_t);
}  // namespace p2de
