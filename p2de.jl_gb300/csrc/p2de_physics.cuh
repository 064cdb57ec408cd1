// Compressible-Euler point functions on the device, following
// src/math/compressible_Navier_Stokes.jl (Dim2 unless noted). The FP64
// instantiation keeps the reference's association order; the FP32 one is used
// only by the mixed-precision flux-differencing terms.
#pragma once

#include <cuda_runtime.h>
#include <math.h>

namespace p2de {

template <typename T>
struct Gas {
  T gamma;   // gamma
  T gm1;     // gamma - 1.0 (computed once on the host as the reference does at run time)
  T two_gm1; // 2 * (gamma - 1)
};

// pfun (:24-28)
template <typename T>
__device__ __forceinline__ T pfun(const Gas<T>& g, T rho, T rhou, T rhov, T E) {
  return g.gm1 * (E - T(0.5) * (rhou * rhou + rhov * rhov) / rho);
}

// rhoe_ufun (:75-78)
template <typename T>
__device__ __forceinline__ T rhoe_ufun(T rho, T rhou, T rhov, T E) {
  return E - T(0.5) * (rhou * rhou + rhov * rhov) / rho;
}

// FP32 logarithmic mean (aL - aR)/(log aL - log aR) by the stable expansion of
// Ismail & Roe, J. Comput. Phys. 228 (2009) 5410-5436, Appendix B:
// xi = aL/aR, f = (xi-1)/(xi+1), u = f^2,
// F = log(xi)/(2f) = 1 + u/3 + u^2/5 + u^3/7 (u < 1e-2), logmean = (aL+aR)/(2F).
// FP32 log(aL) - log(aR) cancels when aL ~ aR, so the logs of the ratio are used.
__device__ __forceinline__ float logmean_f32(float aL, float aR) {
  float xi = aL / aR;
  float f = (xi - 1.0f) / (xi + 1.0f);
  float u = f * f;
  float F;
  if (u < 1.0e-2f) {
    F = 1.0f + u * (1.0f / 3.0f + u * (1.0f / 5.0f + u * (1.0f / 7.0f)));
  } else {
    F = logf(xi) / (2.0f * f);
  }
  return (aL + aR) / (2.0f * F);
}

// fS(Dim2) in FP32 with the Ismail-Roe log mean; UL/UR = (rho, u, v, beta).
__device__ __forceinline__ void fS_f32(const Gas<float>& g, const float* UL, const float* UR, float* Fx, float* Fy) {
  float rholog = logmean_f32(UL[0], UR[0]);
  float betalog = logmean_f32(UL[3], UR[3]);
  float rhoavg = 0.5f * (UL[0] + UR[0]);
  float uavg = 0.5f * (UL[1] + UR[1]);
  float vavg = 0.5f * (UL[2] + UR[2]);
  float unorm = UL[1] * UR[1] + UL[2] * UR[2];
  float pa = rhoavg / (UL[3] + UR[3]);
  float f4aux = rholog / (g.two_gm1 * betalog) + pa + 0.5f * rholog * unorm;
  float FxS1 = rholog * uavg;
  float FxS3 = FxS1 * vavg;
  float FyS1 = rholog * vavg;
  Fx[0] = FxS1;
  Fx[1] = FxS1 * uavg + pa;
  Fx[2] = FxS3;
  Fx[3] = f4aux * uavg;
  Fy[0] = FyS1;
  Fy[1] = FxS3;
  Fy[2] = FyS1 * vavg + pa;
  Fy[3] = f4aux * vavg;
}

// Julia min/max semantics on Float64: NaN propagates, -0.0 < 0.0.
__device__ __forceinline__ double jmin(double x, double y) {
  if (isnan(x) || isnan(y)) return __longlong_as_double(0x7ff8000000000000LL);
  if (x == y) return signbit(x) ? x : y;
  return x < y ? x : y;
}
__device__ __forceinline__ double jmax(double x, double y) {
  if (isnan(x) || isnan(y)) return __longlong_as_double(0x7ff8000000000000LL);
  if (x == y) return signbit(x) ? y : x;
  return x > y ? x : y;
}

}  // namespace p2de
