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

// wavespeed_estimate(Dim2, U, n) (:59-62) -> Dim1 form (:18-22, :48-52) on
// Un = (rho, n1*rhou + n2*rhov, E). Only n enters through un.
template <typename T>
__device__ __forceinline__ T wavespeed_un(const Gas<T>& g, T rho, T un, T E) {
  T p = g.gm1 * (E - T(0.5) * (un * un) / rho);
  return fabs(un / rho) + sqrt(g.gamma * p / rho);
}

template <typename T>
__device__ __forceinline__ T wavespeed(const Gas<T>& g, const T* U, T n1, T n2) {
  return wavespeed_un(g, U[0], n1 * U[1] + n2 * U[2], U[3]);
}

// fluxes(Dim2) (:175-194): fx[0..3], fy[0..3]
template <typename T>
__device__ __forceinline__ void fluxes(const Gas<T>& g, const T* U, T* fx, T* fy) {
  T rho = U[0], rhou = U[1], rhov = U[2], E = U[3];
  T p = pfun(g, rho, rhou, rhov, E);
  T u = rhou / rho;
  T v = rhov / rho;
  T rhouv = rho * u * v;
  T Ep = E + p;
  fx[0] = rhou;
  fx[1] = rhou * u + p;
  fx[2] = rhouv;
  fx[3] = u * Ep;
  fy[0] = rhov;
  fy[1] = rhouv;
  fy[2] = rhov * v + p;
  fy[3] = v * Ep;
}

// logmean(aL, aR, logL, logR) (:307-321), the reference's series and threshold.
__device__ __forceinline__ double logmean_ref(double aL, double aR, double logL, double logR) {
  double da = aR - aL;
  double aavg = 0.5 * (aR + aL);
  double f = da / aavg;
  double v = f * f;
  if (fabs(f) < 1e-4) {
    return aavg * (1.0 + v * (-0.2 - v * (0.0512 - v * 0.026038857142857)));
  }
  return -da / (logL - logR);
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

// fS(Dim2) (:220-249) with logs precomputed per node (FP64, reference formula).
// UL/UR = (rho, u, v, beta, log rho, log beta). Writes Fx[4], Fy[4].
__device__ __forceinline__ void fS_f64(const Gas<double>& g, const double* UL, const double* UR, double* Fx,
                                       double* Fy) {
  double rholog = logmean_ref(UL[0], UR[0], UL[4], UR[4]);
  double betalog = logmean_ref(UL[3], UR[3], UL[5], UR[5]);
  double rhoavg = 0.5 * (UL[0] + UR[0]);
  double uavg = 0.5 * (UL[1] + UR[1]);
  double vavg = 0.5 * (UL[2] + UR[2]);
  double unorm = UL[1] * UR[1] + UL[2] * UR[2];
  double pa = rhoavg / (UL[3] + UR[3]);
  double f4aux = rholog / (g.two_gm1 * betalog) + pa + 0.5 * rholog * unorm;
  double FxS1 = rholog * uavg;
  double FxS3 = FxS1 * vavg;
  double FyS1 = rholog * vavg;
  Fx[0] = FxS1;
  Fx[1] = FxS1 * uavg + pa;
  Fx[2] = FxS3;
  Fx[3] = f4aux * uavg;
  Fy[0] = FyS1;
  Fy[1] = FxS3;
  Fy[2] = FyS1 * vavg + pa;
  Fy[3] = f4aux * vavg;
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
