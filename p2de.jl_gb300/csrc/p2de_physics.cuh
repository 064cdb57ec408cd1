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

// The parts of fS(Dim2) in FP32 that both directions share (Ismail-Roe log mean);
// UL/UR = (rho, u, v, beta).
struct FSCommonF {
  float rholog, uavg, vavg, pa, f4aux;
};
__device__ __forceinline__ FSCommonF fS_common_f32(const Gas<float>& g, const float* UL, const float* UR) {
  FSCommonF c;
  c.rholog = logmean_f32(UL[0], UR[0]);
  const float betalog = logmean_f32(UL[3], UR[3]);
  const float rhoavg = 0.5f * (UL[0] + UR[0]);
  c.uavg = 0.5f * (UL[1] + UR[1]);
  c.vavg = 0.5f * (UL[2] + UR[2]);
  const float unorm = fmaf(UL[1], UR[1], UL[2] * UR[2]);
  c.pa = rhoavg / (UL[3] + UR[3]);
  c.f4aux = fmaf(0.5f * c.rholog, unorm, c.rholog / (g.two_gm1 * betalog) + c.pa);
  return c;
}

// fS(Dim2) in FP32, both directions
__device__ __forceinline__ void fS_f32(const Gas<float>& g, const float* UL, const float* UR, float* Fx, float* Fy) {
  const FSCommonF c = fS_common_f32(g, UL, UR);
  const float FxS1 = c.rholog * c.uavg;
  const float FxS3 = FxS1 * c.vavg;
  const float FyS1 = c.rholog * c.vavg;
  Fx[0] = FxS1;
  Fx[1] = fmaf(FxS1, c.uavg, c.pa);
  Fx[2] = FxS3;
  Fx[3] = c.f4aux * c.uavg;
  Fy[0] = FyS1;
  Fy[1] = FxS3;
  Fy[2] = fmaf(FyS1, c.vavg, c.pa);
  Fy[3] = c.f4aux * c.vavg;
}

// the x (ax = 0) or y (ax = 1) flux of fS_f32 alone (axis-aligned elements)
__device__ __forceinline__ void fS_f32_axis(const Gas<float>& g, const float* UL, const float* UR, int ax, float* F) {
  const FSCommonF c = fS_common_f32(g, UL, UR);
  const float un = ax ? c.vavg : c.uavg;
  const float F0 = c.rholog * un;
  const float Ft = (c.rholog * c.uavg) * c.vavg;
  const float Fn = fmaf(F0, un, c.pa);
  F[0] = F0;
  F[1] = ax ? Ft : Fn;
  F[2] = ax ? Fn : Ft;
  F[3] = c.f4aux * un;
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
