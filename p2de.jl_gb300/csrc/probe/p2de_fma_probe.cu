// Roofline denominator probe for the benchmark (built as libp2de_probe.so, not part of the
// solver library): FMA throughput of this GPU (independent FMA chains per thread, no memory
// traffic but one store per thread), in FP64 or FP32. Returns 0 on success, 3 on a CUDA
// error, 4 when the output buffer cannot be allocated.
#include <cuda_runtime.h>
#include <stdint.h>

enum { PROBE_OK = 0, PROBE_ERR_ARG = 1, PROBE_ERR_CUDA = 3, PROBE_ERR_OOM = 4 };

namespace {

template <typename T>
__global__ void k_fma_chains(T* out, int iters, T a, T b) {
  T x0 = threadIdx.x * (T)1e-3, x1 = x0 + (T)1, x2 = x0 + (T)2, x3 = x0 + (T)3;
  T x4 = x0 + (T)4, x5 = x0 + (T)5, x6 = x0 + (T)6, x7 = x0 + (T)7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b);
    x1 = fma(x1, a, b);
    x2 = fma(x2, a, b);
    x3 = fma(x3, a, b);
    x4 = fma(x4, a, b);
    x5 = fma(x5, a, b);
    x6 = fma(x6, a, b);
    x7 = fma(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

template <typename T>
int run(int device, int iters, double* tflops) {
  if (cudaSetDevice(device) != cudaSuccess) return PROBE_ERR_CUDA;
  cudaDeviceProp p;
  if (cudaGetDeviceProperties(&p, device) != cudaSuccess) return PROBE_ERR_CUDA;
  const int threads = 256, blocks = p.multiProcessorCount * 8;
  T* out = nullptr;
  if (cudaMalloc(&out, sizeof(T) * blocks * threads) != cudaSuccess) return PROBE_ERR_OOM;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_fma_chains<T><<<blocks, threads>>>(out, iters / 4, (T)0.999999, (T)1e-7);  // warm-up
  cudaEventRecord(e0);
  k_fma_chains<T><<<blocks, threads>>>(out, iters, (T)0.999999, (T)1e-7);
  cudaEventRecord(e1);
  cudaError_t e = cudaEventSynchronize(e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (e != cudaSuccess || ms <= 0) return PROBE_ERR_CUDA;
  *tflops = 2.0 * 8.0 * (double)iters * blocks * threads / (ms * 1e-3) / 1e12;
  return PROBE_OK;
}

}  // namespace

extern "C" int p2de_probe_fma_peak(int device, int32_t fp64, double* tflops) {
  if (!tflops) return PROBE_ERR_ARG;
  return fp64 ? run<double>(device, 4096, tflops) : run<float>(device, 16384, tflops);
}
