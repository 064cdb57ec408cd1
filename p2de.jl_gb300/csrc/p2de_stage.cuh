// Stage kernels for tensor-product GLL elements of N1D = N+1 nodes per line.
//
// Stage kernel A (one block = E consecutive elements; every phase is a flat loop
// over (element, item) so that the FP64 pipe, the bottleneck here, always issues
// full warps):
//   low-order graph-viscosity RHS      low_order_graph_viscosity.jl:4-41
//   high-order ES flux differencing    flux_differencing.jl:4-37
//   subcell bounds and cell entropy    subcell.jl:163-349, 462-744; limiter_utils.jl:66-132
// Stage kernel B: symmetrization across element faces (subcell.jl:418-456), limited
// subcell fluxes and rhsU (subcell.jl:841-924), SSP-RK3 stage combination
// (SSPRK33.jl:127-135) and the per-stage positivity record.
//
// GB300 executes FP64 at 2 FMA/clk/SM, 1/58 of its FP32 rate, so these kernels are
// bound by their FP64 instruction count. The arithmetic follows the reference's
// formulas and association order, with these departures, each within a few units in
// the last place of the reference's value:
//  * a quotient by the same denominator is a multiplication by one reciprocal
//    (1/rho per node, 1/J per element, 1/(2a) per quadratic; 1/(wq J) is (1/J)(1/wq));
//  * the entropy log(p / rho^gamma) of the entropy variables is log p - gamma log rho;
//  * the log mean (compressible_Navier_Stokes.jl:307-321) takes one quotient: the
//    branch test |da/aavg| < 1e-4 is made as |da| < 1e-4 |aavg|, then da is divided by
//    aavg (series branch) or by log(aL) - log(aR); the two log means of a two-point
//    flux share one reciprocal for their quotients;
//  * pa and rholog/(2(gamma-1) betalog) of fS share one reciprocal;
//  * min/max are fmin/fmax, which differ from Julia's min/max only for NaN operands
//    (a NaN state is reported through the status word instead);
//  * on axis-aligned elements (sxJ = ryJ = 0) the terms the reference multiplies by an
//    exact zero are not formed.
// For LGL collocation two parts of the reference's computation are identities up to
// rounding and are not evaluated:
//  * the entropy projection of face values, u_vfun(v_ufun(U)) (rhs.jl:242-252; the
//    reference itself notes "we can skip LGL instead of applying identity", rhs.jl:265);
//  * the hybridized face-volume pairs (Nq+f, fq2q[f]) of Srsh_nnz, whose contributions
//    to QF1[Nq+f] and QF1[fq2q[f]] cancel when MinvVhT (init.jl:171) lifts QF1[Nq+f]
//    back onto node fq2q[f].
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "p2de_args.h"
#include "p2de_physics.cuh"
#include "p2de_tables.h"

namespace p2de {

__host__ __device__ constexpr int cmax(int a, int b) { return a > b ? a : b; }
__host__ __device__ constexpr int cmin(int a, int b) { return a < b ? a : b; }

template <int N1D>
struct Cfg {
  static constexpr int n = N1D;
  static constexpr int Nq = n * n;
  static constexpr int Nfp = 4 * n;
  static constexpr int NPL = 2 * n * (n - 1);
  static constexpr int NPH = n * n * (n - 1);
  static constexpr int NSF = n * (n + 1);  // subcell faces per direction = Nq + N1D
  static constexpr int NEV = 4 * Nq;       // bound evaluations per element
  static constexpr int E = (64 / Nq) > 0 ? (64 / Nq) : 1;  // default elements per block
  static constexpr int THREADS = 128;
  static constexpr int SCR = cmax(cmax(NPL * 9, NPH * 8), 16 * NSF);
  // shared-memory doubles per element, kernel A; regions whose lifetimes (phases) do not
  // overlap share storage
  static constexpr int O_GEO = 0;                  // 16: J, rxJ, sxJ, ryJ, syJ, |gr|, nr, |gs|, ns, 1/J,
                                                   // FP32 copies (12-14), blending factor (15)
  static constexpr int O_U = O_GEO + 16;           // 4 Nq
  static constexpr int O_PRIM = O_U + 4 * Nq;      // 6 Nq: primitives (P1-P6); uL[4], Lrhoe, 4dt/(wq J) (P8-P9)
  static constexpr int O_FLUX = O_PRIM + 6 * Nq;   // 8 Nq: nodal fluxes (P1-P4)
  static constexpr int O_RXYH = O_FLUX;            //       high-order rhsxy (P7-P8)
  static constexpr int O_EV = O_FLUX;              //       bound evaluations NEV = 4 Nq (P9-P10), then vq (P11)
  static constexpr int O_L = O_FLUX + 4 * Nq;      //       subcell factors 2 NSF (P10-P12)
  static constexpr int O_MISC = O_L + 2 * NSF;     //       4 (P11)
  static constexpr int O_WS = O_FLUX + 8 * Nq;     // 2 Nq: wavespeeds (P1-P4); wq J, 1/(wq J) (P5-P8)
  static constexpr int O_RXYL = O_WS + 2 * Nq;     // 8 Nq (P3-P8)
  static constexpr int O_RHSL = O_RXYL + 8 * Nq;   // 4 Nq (P5-P8); density-bound Lrho, rho/2 (P8-P9)
  static constexpr int O_LAMI = O_RHSL + 4 * Nq;   // Nq (P3-P5)
  static constexpr int O_BFL = O_LAMI + Nq;        // 8 Nfp (P4-P8)
  static constexpr int O_BFH = O_BFL + 8 * Nfp;    // 8 Nfp (P4-P8)
  static constexpr int O_LAMB = O_BFH + 8 * Nfp;   // Nfp (P4-P5)
  static constexpr int O_SCR = O_LAMB + Nfp;       // SCR: pair terms (P2-P3, P6-P7), subcell fluxes (P8-P12)
  static_assert(O_MISC + 4 <= O_WS, "limiter data fit the flux region");
  // even, so that every element's block (and its FP32 float4 vectors) is 16-byte aligned
  static constexpr int PER_ELEM_A = (O_SCR + SCR + 1) & ~1;
  static_assert(PER_ELEM_A % 2 == 0 && O_PRIM % 2 == 0, "16-byte alignment of per-element data");
  // plus a block-wide list of bound evaluations that need the quadratic solve
  static constexpr size_t smem_a(int e) { return sizeof(double) * PER_ELEM_A * e + sizeof(int) * (NEV * e + 4); }
  static constexpr size_t SMEM_A = smem_a(E);
  // kernel B
  static constexpr int PER_ELEM_B = 2 * NSF + 16 * NSF + 8 * NSF + 8;
  static constexpr size_t smem_b(int e) { return sizeof(double) * PER_ELEM_B * e; }
  static constexpr size_t SMEM_B = smem_b(E);
  // largest elements-per-block whose kernel-A shared memory fits 224 KB (capped at 32)
  static constexpr int E_MAX_RAW = (int)((224 * 1024 - 64) / (sizeof(double) * PER_ELEM_A + sizeof(int) * NEV));
  static constexpr int E_MAX = E_MAX_RAW < 32 ? E_MAX_RAW : 32;
  static constexpr int FBAR = 16 * NSF;  // per element: [dir][H/L][face][c]
  // EXT instantiations of kernel A: two more doubles per element after the LGL layout,
  // the relaxed bounds' smoothness factor (O_XT) and the Gauss limited flag (O_XT + 1)
  static constexpr int O_XT = PER_ELEM_A;
  static constexpr int PER_ELEM_X = PER_ELEM_A + 2;
  static constexpr size_t smem_x(int e) { return sizeof(double) * PER_ELEM_X * e + sizeof(int) * (NEV * e + 4); }
  static_assert((224 * 1024 - 64) / (sizeof(double) * PER_ELEM_X + sizeof(int) * NEV) >= (size_t)E_MAX,
                "the EXT layout fits every elements-per-block value of the LGL one");
  // GaussCollocation (kernel A with GAUSS): after those, the projected face states, their
  // primitives, theta, the face rows of QF1 and the volume-face pair terms
  static constexpr int O_UF = PER_ELEM_X;                // 4 Nfp
  static constexpr int O_PF = O_UF + 4 * Nfp;       // 6 Nfp
  static constexpr int O_TH = O_PF + 6 * Nfp;       // Nfp
  static constexpr int O_QFF = O_TH + Nfp;          // 8 Nfp
  static constexpr int O_FPT = O_QFF + 8 * Nfp;     // 8 Nfp n: pair (face f, line node a) at f n + a
  static constexpr int PER_ELEM_G = (O_FPT + 8 * Nfp * n + 1) & ~1;
  static constexpr size_t smem_g(int e) { return sizeof(double) * PER_ELEM_G * e + sizeof(int) * (NEV * e + 4); }
  static constexpr int E_G = (64 / Nq) > 0 ? (64 / Nq) : 1;
  static constexpr int E_MAX_G_RAW = (int)((224 * 1024 - 64) / (sizeof(double) * PER_ELEM_G + sizeof(int) * NEV));
  static constexpr int E_MAX_G = E_MAX_G_RAW < 32 ? E_MAX_G_RAW : 32;
  static_assert(O_UF % 2 == 0 && E_G <= E_MAX_G, "Gauss layout");
  // the face projection kernel: U and v(U) per node
  static constexpr int PER_ELEM_P = 8 * Nq;
  static constexpr size_t smem_p(int e) { return sizeof(double) * PER_ELEM_P * e; }
};

// U + dt rhsL, the low-order update (one form everywhere, so values agree bitwise)
__device__ __forceinline__ double low_update(double u, double dt, double r) { return fma(dt, r, u); }

// 1/x: for |x| in [2^-1022, 2^1022) (a normal reciprocal) two Newton-Raphson steps
// y <- y + y (1 - x y) from the hardware's approximate reciprocal (rcp.approx.ftz.f64),
// each residual formed by an FMA; the result is the correctly rounded 1/x unless 1/x lies
// within about 2^-88 relative of a rounding tie (the same bits as __drcp_rn on 4M random
// arguments), in 5 FP64 instructions against 6. Other x (0, subnormal, huge, inf, NaN) take
// __drcp_rn.
__device__ __forceinline__ double rcp(double x) {
  const unsigned long long a = (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffULL;
  if (a - 0x0010000000000000ULL >= 0x7fc0000000000000ULL) return __drcp_rn(x);
  double y;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
  double e = fma(-x, y, 1.0);
  y = fma(y, e, y);
  e = fma(-x, y, 1.0);
  return fma(y, e, y);
}

// Natural logarithm by the table-driven method of P. T. P. Tang ("Table-driven implementation
// of the logarithm function in IEEE floating-point arithmetic", ACM TOMS 16(4), 1990):
// x = 2^k m with m in [sqrt(1/2), sqrt(2)), F = m rounded to a multiple of 1/256 (table
// entry j), r = (m - F) / F (m - F exact), log x = k log 2 + log F + log(1 + r), the last
// by its Taylor polynomial to r^6 (|r| < 2^-8.5: the omitted terms are below 2^-56 of the
// result). 15 FP64 instructions against 31 for log(); within one unit in the last place of
// the correctly rounded value (checked against an extended-precision log on 4M arguments
// from 1e-9 to 2e8 and around 1), like log(). Positive normal finite x; anything else
// goes to log().
__device__ __forceinline__ double log_fast(double x, const OpTable& op) {
  const long long b = __double_as_longlong(x);
  if ((unsigned long long)(b - 0x0010000000000000LL) >= 0x7fe0000000000000ULL) return log(x);
  long long k = (b >> 52) - 1023;
  long long mb = (b & 0x000fffffffffffffLL) | 0x3ff0000000000000LL;  // m in [1, 2)
  if (((mb >> 44) & 0xff) >= 106) {  // m >= 1 + 106/256: use m/2 in [0.707, 1)
    mb -= 0x0010000000000000LL;
    k += 1;
  }
  const double m = __longlong_as_double(mb);
  const double t = m + 0x1p44;  // m rounded to a multiple of 2^-8 in the low mantissa bits
  const int j = (int)(__double_as_longlong(t) & 0x1ff);
  const double F = t - 0x1p44;
  const double* T = op.logtab[j - kLogTabLo];
  const double r = (m - F) * T[0];
  double q = fma(r, -1.0 / 6.0, 1.0 / 5.0);
  q = fma(q, r, -0.25);
  q = fma(q, r, 1.0 / 3.0);
  q = fma(q, r, -0.5);
  const double p = fma(r * r, q, r);
  // (double)k without a conversion: 1.5 2^52 + k in the bits of 1.5 2^52, minus 1.5 2^52
  const double kd = __longlong_as_double(0x4338000000000000LL + k) - 0x1.8p52;
  const double hi = fma(kd, op.ln2_hi, T[1]);
  const double lo = fma(kd, op.ln2_lo, T[2]);
  return hi + (p + lo);
}

// Geometry factor q of an element from gg = (J, rxJ, sxJ, ryJ, syJ): slots 0-4 copy gg,
// then |gr|, nr (2), |gs|, ns (2), 1/J; slots 12-14 hold FP32 rxJ, sxJ, ryJ, syJ, 1/J
// (q = 12..16 write float q-12). Used by the per-element table and by P0 without one.
__device__ __forceinline__ void geom_factor(const double* gg, int q, double* G) {
  if (q < 5) {
    G[q] = gg[q];
  } else if (q < 11) {
    const bool r = q < 8;  // r-normal: (rxJ, ryJ); s-normal: (sxJ, syJ)
    const double g1 = r ? gg[1] : gg[2], g2 = r ? gg[3] : gg[4];
    const double gn = sqrt(g1 * g1 + g2 * g2);
    const int j = (q - 5) % 3;
    G[q] = j == 0 ? gn : (j == 1 ? g1 : g2) / gn;
  } else if (q == 11) {
    G[11] = __drcp_rn(gg[0]);
  } else {
    float* Gf = reinterpret_cast<float*>(G + 12);
    Gf[q - 12] = q < 16 ? (float)gg[q - 11] : (float)__drcp_rn(gg[0]);
  }
}
constexpr int kGeomFactors = 17;  // q = 0..16
constexpr int kGeomStride = 16;   // doubles per element in the table

// ordered 64-bit key of a double (monotone for non-NaN values), for atomicMin
__device__ __forceinline__ long long order_key(double x) {
  long long b = __double_as_longlong(x);
  return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}

// wavespeed_estimate (compressible_Navier_Stokes.jl:48-62) with 1/rho given
// (E - 0.5*(un*un)*rr as one FMA: the factor 0.5 is exact, so the value is unchanged;
// gamma*(gamma-1) is one constant)
__device__ __forceinline__ double wavespeed_r(const Gas<double>& g, double rr, double un, double E) {
  double pe = fma(-0.5, (un * un) * rr, E);
  return fabs(un * rr) + sqrt((g.gamma * g.gm1) * pe * rr);
}

// x with its sign flipped when sign < 0 (integer pipe): q + signed(x, s) is q + s*x for s = +-1
__device__ __forceinline__ double signed_by(double x, int sign) {
  return __longlong_as_double(__double_as_longlong(x) ^ (sign < 0 ? (long long)0x8000000000000000ULL : 0LL));
}

__device__ __forceinline__ float signed_by(float x, int sign) {
  return __int_as_float(__float_as_int(x) ^ (sign < 0 ? (int)0x80000000u : 0));
}

// x == +-0 by its bits (integer pipe instead of the FP64 pipe)
__device__ __forceinline__ bool is_zero_bits(double x) { return (__double_as_longlong(x) << 1) == 0; }

// min of two values in [0, Inf] (either zero's sign) or NaN, by their magnitude bits: a
// NaN loses against any number, as with fmin; the result of a zero is +0
__device__ __forceinline__ double min_nonneg_bits(double a, double b) {
  long long x = __double_as_longlong(a) & 0x7fffffffffffffffLL, y = __double_as_longlong(b) & 0x7fffffffffffffffLL;
  return __longlong_as_double(x < y ? x : y);
}

// fluxes(Dim2) (:175-194) with 1/rho given
__device__ __forceinline__ void fluxes_r(const Gas<double>& g, const double* U, double rr, double* fx, double* fy) {
  double rho = U[0], rhou = U[1], rhov = U[2], E = U[3];
  double p = g.gm1 * fma(-0.5, (rhou * rhou + rhov * rhov) * rr, E);
  double u = rhou * rr, v = rhov * rr;
  double rhouv = rho * u * v;
  double Ep = E + p;
  fx[0] = rhou;
  fx[1] = rhou * u + p;
  fx[2] = rhouv;
  fx[3] = u * Ep;
  fy[0] = rhov;
  fy[1] = rhouv;
  fy[2] = rhov * v + p;
  fy[3] = v * Ep;
}

// the x (xaxis) or y flux of fluxes_r alone
__device__ __forceinline__ void flux_axis_r(const Gas<double>& g, const double* U, double rr, bool xaxis, double* f) {
  double rho = U[0], rhou = U[1], rhov = U[2], E = U[3];
  double p = g.gm1 * fma(-0.5, (rhou * rhou + rhov * rhov) * rr, E);
  double u = rhou * rr, v = rhov * rr;
  double rhouv = rho * u * v;
  double Ep = E + p;
  double mn = xaxis ? rhou : rhov, un = xaxis ? u : v;
  double fn = mn * un + p;
  f[0] = mn;
  f[1] = xaxis ? fn : rhouv;
  f[2] = xaxis ? rhouv : fn;
  f[3] = un * Ep;
}

// logmean (compressible_Navier_Stokes.jl:307-321), series branch, for x = da/aavg
__device__ __forceinline__ double logmean_series(double aavg, double x) {
  double v = x * x;
  return aavg * (1.0 + v * (-0.2 - v * (0.0512 - v * 0.026038857142857)));
}

// The parts of fS(Dim2) (:220-249) that both flux directions share: the log means, the
// averages, pa and f4aux. UL/UR = (rho, u, v, beta, log rho, log beta). The quotients of
// the two log means (logmean_1div) share one reciprocal: da_r/den_r = da_r den_b/(den_r den_b).
struct FSCommon {
  double rholog, uavg, vavg, pa, f4aux;
};
__device__ __forceinline__ FSCommon fS_common(const Gas<double>& g, const double* UL, const double* UR) {
  const double da_r = UR[0] - UL[0], av_r = 0.5 * (UR[0] + UL[0]);
  const bool ser_r = fabs(da_r) < 1e-4 * fabs(av_r);
  const double den_r = ser_r ? av_r : (UL[4] - UR[4]);
  const double da_b = UR[3] - UL[3], av_b = 0.5 * (UR[3] + UL[3]);
  const bool ser_b = fabs(da_b) < 1e-4 * fabs(av_b);
  const double den_b = ser_b ? av_b : (UL[5] - UR[5]);
  const double rd = rcp(den_r * den_b);
  const double x_r = da_r * (den_b * rd), x_b = da_b * (den_r * rd);
  FSCommon c;
  c.rholog = ser_r ? logmean_series(av_r, x_r) : -x_r;
  const double betalog = ser_b ? logmean_series(av_b, x_b) : -x_b;
  const double rhoavg = 0.5 * (UL[0] + UR[0]);
  c.uavg = 0.5 * (UL[1] + UR[1]);
  c.vavg = 0.5 * (UL[2] + UR[2]);
  const double unorm = fma(UL[1], UR[1], UL[2] * UR[2]);
  const double d1 = UL[3] + UR[3];
  const double d2 = g.two_gm1 * betalog;
  const double r12 = rcp(d1 * d2);
  c.pa = rhoavg * d2 * r12;
  c.f4aux = fma(c.rholog * d1, r12, c.pa) + (0.5 * c.rholog) * unorm;
  return c;
}

// fS(Dim2) (:220-249), both directions
__device__ __forceinline__ void fS_fast(const Gas<double>& g, const double* UL, const double* UR, double* Fx,
                                        double* Fy) {
  const FSCommon c = fS_common(g, UL, UR);
  const double FxS1 = c.rholog * c.uavg;
  const double FxS3 = FxS1 * c.vavg;
  const double FyS1 = c.rholog * c.vavg;
  Fx[0] = FxS1;
  Fx[1] = fma(FxS1, c.uavg, c.pa);
  Fx[2] = FxS3;
  Fx[3] = c.f4aux * c.uavg;
  Fy[0] = FyS1;
  Fy[1] = FxS3;
  Fy[2] = fma(FyS1, c.vavg, c.pa);
  Fy[3] = c.f4aux * c.vavg;
}

// the x (ax = 0) or y (ax = 1) flux of fS_fast alone, with the same operations for each
// component: on axis-aligned elements a pair on an r-line needs only the x flux and a pair
// on an s-line only the y flux, and one instruction stream serves both
__device__ __forceinline__ void fS_axis(const Gas<double>& g, const double* UL, const double* UR, int ax,
                                        double* F) {
  const FSCommon c = fS_common(g, UL, UR);
  const double un = ax ? c.vavg : c.uavg;
  const double F0 = c.rholog * un;                 // FxS1 or FyS1
  const double Ft = (c.rholog * c.uavg) * c.vavg;  // FxS3: Fx[2] and Fy[1]
  const double Fn = fma(F0, un, c.pa);             // Fx[1] or Fy[2]
  F[0] = F0;
  F[1] = ax ? Ft : Fn;
  F[2] = ax ? Fn : Ft;
  F[3] = c.f4aux * un;
}

// limiter_utils.jl:108-132 for a finite Lrhoe
__device__ __forceinline__ double rhoe_quadratic_solve(const double* U, const double* P, double Lrhoe,
                                                       double ZEROTOL) {
  // limiter_utils.jl:141-146
  double a = P[0] * P[3] - 1.0 / 2.0 * (P[1] * P[1] + P[2] * P[2]);
  double b = U[3] * P[0] + U[0] * P[3] - U[1] * P[1] - U[2] * P[2] - P[0] * Lrhoe;
  double c = U[3] * U[0] - 1.0 / 2.0 * (U[1] * U[1] + U[2] * U[2]) - U[0] * Lrhoe;
  double l = 1.0;
  double disc = b * b - 4.0 * a * c;
  if (disc >= 0.0) {
    double sq = sqrt(disc);
    double r2a = rcp(2.0 * a);
    double r1 = (-b + sq) * r2a;
    double r2 = (-b - sq) * r2a;
    if (r1 > ZEROTOL && r2 > ZEROTOL) {
      l = fmin(r1, r2);
    } else if (r1 > ZEROTOL && r2 < -ZEROTOL) {
      l = r1;
    } else if (r2 > ZEROTOL && r1 < -ZEROTOL) {
      l = r2;
    }
  }
  return l;
}

// Density part of limiting_param_bound_rho_rhoe (limiter_utils.jl:82-92) for the
// positivity bounds Lrho = zeta*rhoL and Urho = 0 (the Lphi slot under the reference's
// destructuring, limiter_utils.jl:66-70) or Inf.
// Density part of limiting_param_bound_rho_rhoe for [Lrho, Urho]. upper0: Urho = 0 (the
// Lphi slot under the reference's destructuring). With upper0, U0 > 0 and U0 + P0 not below Lrho, the factor
// fmin(1, fmax((0 - U0)/P0, 0)) is 0 for P0 >= +0 and 1 for P0 <= -0 with |P0| < U0/2
// (the quotient is then above 2), so it is set without the division; hU0 = U0/2.
__device__ __forceinline__ double density_bound(double U0, double P0, double Lrho, double Urho, bool upper0,
                                                double hU0) {
  double l = 1.0;
  double up = U0 + P0;
  bool lo = up < Lrho, hi = up > Urho;
  if (lo || hi) {
    if (!lo && upper0 && __double_as_longlong(U0) > 0) {
      if (!signbit(P0)) return 0.0;
      if (-P0 < hU0) return 1.0;
    }
    double rP = rcp(P0);
    if (lo) l = fmax((Lrho - U0) * rP, 0.0);
    if (hi) l = fmin(l, fmax((Urho - U0) * rP, 0.0));
  }
  return l;
}

// fS(::KPP{Dim2}) (KPP.jl:25-38), psi = (-cos u, sin u): the scalar fluxes in component 0
__device__ __forceinline__ void fS_kpp(double uL, double uR, double* Fx, double* Fy) {
  if (fabs(uR - uL) < 1e-12) {
    Fx[0] = 0.5 * (sin(uL) + sin(uR));
    Fy[0] = 0.5 * (cos(uL) + cos(uR));
  } else {
    Fx[0] = (-cos(uR) - -cos(uL)) / (uR - uL);
    Fy[0] = (sin(uR) - sin(uL)) / (uR - uL);
  }
#pragma unroll
  for (int c = 1; c < 4; ++c) Fx[c] = Fy[c] = 0.0;
}

// find_alpha(::CompressibleIdealGas) (low_order_graph_viscosity.jl:316-340): doubling, then
// 50 halvings toward the alpha with alpha ui - uitilde of positive density and rhoe
__device__ __forceinline__ double find_alpha(const double* ui, const double* ut, double POSTOL) {
  auto ok = [&](double al) {
    double q[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) q[c] = al * ui[c] - ut[c];
    return q[0] > POSTOL && q[3] - 0.5 * (q[1] * q[1] + q[2] * q[2]) / q[0] > POSTOL;
  };
  double alphaL = 0.0, alphaR = 1.0;
  for (int guard = 0; guard < 1100 && !ok(alphaR); ++guard) alphaR = 2 * alphaR;
  for (int iter = 0; iter < 50; ++iter) {
    const double alphaM = (alphaL + alphaR) / 2;
    if (ok(alphaM))
      alphaR = alphaM;
    else
      alphaL = alphaM;
  }
  return alphaR;
}

// s_modified_ufun (compressible_Navier_Stokes.jl:80-85): phi = rhoe rho^(-gamma), with
// rhoe_ufun written as the reference writes it
__device__ __forceinline__ double s_modified(double rho, double rhou, double rhov, double E, double gamma) {
  const double rhoe = E - 0.5 * (rhou * rhou + rhov * rhov) / rho;
  return rhoe * pow(rho, -gamma);
}

// initialize_s_modified! (subcell.jl:21-35): at t == t0, stage 1, the minimum of
// phi = rhoe rho^(-gamma) over every node (NaN if any is NaN, as Julia's minimum), by one
// block of 1024 threads in a fixed order, so the result does not depend on scheduling.
__device__ __forceinline__ void phi_min_body(const double* Uq, size_t nodes, double gamma, const double* scal,
                                             double t0, double* out) {
  if (scal[S_DONE] != 0.0 || scal[S_T] != t0) return;
  __shared__ double wmin[32];
  __shared__ int wnan[32];
  double m = INFINITY;
  int isn = 0;
  for (size_t i = threadIdx.x; i < nodes; i += blockDim.x) {
    const double* U = Uq + 4 * i;
    const double v = s_modified(U[0], U[1], U[2], U[3], gamma);
    if (isnan(v))
      isn = 1;
    else
      m = fmin(m, v);
  }
  for (int o = 16; o > 0; o >>= 1) {
    m = fmin(m, __shfl_xor_sync(0xffffffffu, m, o));
    isn |= __shfl_xor_sync(0xffffffffu, isn, o);
  }
  if ((threadIdx.x & 31) == 0) {
    wmin[threadIdx.x >> 5] = m;
    wnan[threadIdx.x >> 5] = isn;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
      m = fmin(m, wmin[w]);
      isn |= wnan[w];
    }
    *out = isn ? NAN : m;
  }
}

// limiting_param_bound_phi (limiter_utils.jl:43-50) through bisection (nonlinear_solvers.jl:3-20):
// the l in [0, lpos] closest to lpos, on the grid of 21 halvings, with
// phi(U + l P) >= thr (thr = Lphi - POSTOL); f(0) is assumed, as the reference does. The
// first test, at lpos (phi_at_least), and the 21 halvings after it (bisect_phi_halvings).
__device__ __forceinline__ bool phi_at_least(const double* U, const double* P, double l, double thr, double gamma) {
  return s_modified(U[0] + l * P[0], U[1] + l * P[1], U[2] + l * P[2], U[3] + l * P[3], gamma) >= thr;
}

__device__ __forceinline__ double bisect_phi_halvings(const double* U, const double* P, double lpos, double thr,
                                                      double gamma) {
  double x_valid = 0.0, x_invalid = lpos;
  for (int iter = 0; iter <= 20; ++iter) {
    const double x_new = 0.5 * (x_valid + x_invalid);
    if (phi_at_least(U, P, x_new, thr, gamma))
      x_valid = x_new;
    else
      x_invalid = x_new;
  }
  return x_valid;
}

// Slot s of P9's list of bisections: in the low-order rhsxy region of the block's elements
// (16 Nq ints each, four times an element's evaluations), element s / (16 Nq) first.
template <typename C>
__device__ __forceinline__ int& bisect_slot(double* sm, int PE, int s) {
  constexpr int cap = 16 * C::Nq;
  return reinterpret_cast<int*>(sm + (s / cap) * PE + C::O_RXYL)[s % cap];
}

// v_ufun(::CompressibleIdealGas{Dim2}) (compressible_Navier_Stokes.jl:134-144), with
// s = log(p) - gamma log(rho) for log(p / rho^gamma)
__device__ __forceinline__ void v_ufun_d(const Gas<double>& g, const double* U, double* V) {
  const double p = g.gm1 * (U[3] - 0.5 * (U[1] * U[1] + U[2] * U[2]) / U[0]);
  const double s = log(p) - g.gamma * log(U[0]);
  V[0] = (g.gamma + 1.0 - s) - g.gm1 * U[3] / p;
  V[1] = U[1] * g.gm1 / p;
  V[2] = U[2] * g.gm1 / p;
  V[3] = -U[0] * g.gm1 / p;
}

// v_ufun_d with every operation an explicit round-to-nearest intrinsic: the compiler cannot
// contract it into FMAs, so equal states give bitwise-equal entropy variables wherever it is
// inlined (the interface step compares their jumps with 0)
__device__ __forceinline__ void v_ufun_rn(const Gas<double>& g, const double* U, double* V) {
  const double ke = __ddiv_rn(__dmul_rn(0.5, __dadd_rn(__dmul_rn(U[1], U[1]), __dmul_rn(U[2], U[2]))), U[0]);
  const double p = __dmul_rn(g.gm1, __dsub_rn(U[3], ke));
  const double s = __dsub_rn(log(p), __dmul_rn(g.gamma, log(U[0])));
  V[0] = __dsub_rn(__dsub_rn(__dadd_rn(g.gamma, 1.0), s), __ddiv_rn(__dmul_rn(g.gm1, U[3]), p));
  V[1] = __ddiv_rn(__dmul_rn(U[1], g.gm1), p);
  V[2] = __ddiv_rn(__dmul_rn(U[2], g.gm1), p);
  V[3] = __ddiv_rn(__dmul_rn(-U[0], g.gm1), p);
}

// u_vfun(::CompressibleIdealGas{Dim2}) (:155-163) with rhoe_vfun (:99-104) and s_vfun (:93-97).
// rhoe_vfun = ((gamma-1) / (-vE)^gamma)^(1/(gamma-1)) exp(-s/(gamma-1)) is evaluated as the
// one exponential exp((log(gamma-1) - gamma log(-vE) - s) / (gamma-1)) (the same value to
// about 1e-14 relative; two pow calls fewer); lgm1 = log(gamma - 1).
__device__ __forceinline__ void u_vfun_d(const Gas<double>& g, double lgm1, const double* V, double* U) {
  const double q = (V[1] * V[1] + V[2] * V[2]) / (2.0 * V[3]);
  const double s = g.gamma - V[0] + q;
  const double rhoeV = exp((lgm1 - g.gamma * log(-V[3]) - s) / g.gm1);
  U[0] = -rhoeV * V[3];
  U[1] = rhoeV * V[1];
  U[2] = rhoeV * V[2];
  U[3] = rhoeV * (1.0 - q);
}

// =====================================================================================
// Face projection (GaussCollocation)
// =====================================================================================
// compute_entropyproj_limiting_param!(::GaussCollocation) (filter.jl:6-16), calc_face_values!
// (:28-46), solve_theta!(::NodewiseScaledExtrapolation) (:53-62) with the bounds of
// check_bound_on_face_node (:91-102), then entropy_projection_face_node! (rhs.jl:87-95):
// per face node the values Vf U, Vf v(U) along the line normal to the face, theta by the
// reference's bisection on [0, 1] (theta = 1 without the limiter), and the projected state
// u(sum_a (theta Vf + (1 - theta) Vf_low)_a v_a), written to ufproj and theta.
template <int N1D>
__device__ __forceinline__ void gauss_proj_body(const StageArgs& a, int k0, double* sm) {
  using C = Cfg<N1D>;
  constexpr int n = C::n, Nq = C::Nq, Nfp = C::Nfp, PE = C::PER_ELEM_P;
  if (a.scal[S_DONE] != 0.0) return;
  const OpTable& op = *a.ops;
  const int tid = threadIdx.x, bs = blockDim.x;
  const int Ke = min(a.epb, a.K - k0);
  if (Ke <= 0) return;
  const Gas<double> g{a.gamma, a.gm1, 2.0 * a.gm1};
  for (int w = tid; w < Ke * Nq * 4; w += bs) {
    const int e = w / (Nq * 4), r = w % (Nq * 4);
    sm[e * PE + r] = a.Uq[(size_t)k0 * Nq * 4 + w];
  }
  __syncthreads();
  for (int w = tid; w < Ke * Nq; w += bs) {
    const int e = w / Nq, m = w % Nq;
    v_ufun_d(g, sm + e * PE + 4 * m, sm + e * PE + 4 * Nq + 4 * m);
  }
  __syncthreads();
  const double eps = a.POSTOL, lgm1 = log(a.gm1);
  for (int w = tid; w < Ke * Nfp; w += bs) {
    const int e = w / Nfp, f = w % Nfp, k = k0 + e;
    const int side = f / n, t = f % n;
    const double* ell = (side % 2 == 0) ? op.ellm : op.ellp;
    const int alow = (side % 2 == 0) ? 0 : n - 1;  // the node of Vf_low (fq2q)
    const double* U = sm + e * PE;
    const double* vq = U + 4 * Nq;
    int node[n];
#pragma unroll
    for (int i = 0; i < n; ++i) node[i] = side < 2 ? i + n * t : t + n * i;
    double Uf[4] = {0, 0, 0, 0}, VUf[4] = {0, 0, 0, 0};
#pragma unroll
    for (int i = 0; i < n; ++i) {
      if (ell[i] == 0.0) continue;
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        Uf[c] = Uf[c] + ell[i] * U[4 * node[i] + c];
        VUf[c] = VUf[c] + ell[i] * vq[4 * node[i] + c];
      }
    }
    const double rhoef = Uf[3] - 0.5 * (Uf[1] * Uf[1] + Uf[2] * Uf[2]) / Uf[0];
    auto project = [&](double th, double* vt) {
#pragma unroll
      for (int c = 0; c < 4; ++c) vt[c] = 0.0;
#pragma unroll
      for (int i = 0; i < n; ++i) {
        const double cf = th * ell[i] + (1.0 - th) * (i == alow ? 1.0 : 0.0);
#pragma unroll
        for (int c = 0; c < 4; ++c) vt[c] = vt[c] + cf * vq[4 * node[i] + c];
      }
    };
    // the projected state of theta in ut; returns whether it is well defined and in bounds
    double vt[4], ut[4];
    auto ok = [&](double th) {
      project(th, vt);
      if (!(vt[3] < -eps)) return false;
      u_vfun_d(g, lgm1, vt, ut);
      const double rhoe = ut[3] - 0.5 * (ut[1] * ut[1] + ut[2] * ut[2]) / ut[0];
      return vt[3] < fmin(a.zeta * VUf[3], -eps) && ut[0] > fmax((1 - a.eta) * Uf[0], eps) &&
             ut[0] < (1 + a.eta) * Uf[0] && rhoe > fmax((1 - a.eta) * rhoef, eps) && rhoe < (1 + a.eta) * rhoef;
    };
    double th = 1.0;
    bool have = false;  // ut holds the state of th
    if (a.flags & F_EPROJ) {
      if (ok(1.0)) {
        have = true;
      } else {
        double x_valid = 0.0, x_invalid = 1.0;
        for (int iter = 0; iter <= 20; ++iter) {
          const double x_new = 0.5 * (x_valid + x_invalid);
          if (ok(x_new))
            x_valid = x_new;
          else
            x_invalid = x_new;
        }
        th = x_valid;
      }
    }
    if (!have) {
      project(th, vt);
      u_vfun_d(g, lgm1, vt, ut);
    }
#pragma unroll
    for (int c = 0; c < 4; ++c) a.ufproj[((size_t)k * Nfp + f) * 4 + c] = ut[c];
    a.theta[((size_t)(a.nstage - 1) * a.K + k) * Nfp + f] = th;
  }
}

// enforce_ES_subcell_interface!(::Dim2, ::GaussCollocation) (subcell.jl:759-823) with
// solve_l_es_interface! (:811-817) on the factors before symmetrization: every boundary
// subcell face (one per face node) takes the largest l on the bisection grid of
// [0, min(L, L_partner)] with l dvfH + (1 - l) dvfL <= dpsi, dv and dpsi the jumps of v and
// psi at the face nodes' volume nodes, f* = BF / B on the face's axis. In the order of one
// thread (elements ascending; x faces by line, lower face first, then y faces) the face
// that comes first reads its partner's old factor and the second one the first's new
// one; each pair is done by the item of its first face.
template <int N1D>
__device__ __forceinline__ void es_interface_body(const StageArgs& a, long long w) {
  using C = Cfg<N1D>;
  constexpr int n = C::n, Nq = C::Nq, Nfp = C::Nfp, NSF = C::NSF;
  if (a.scal[S_DONE] != 0.0) return;
  if (w >= (long long)a.K * Nfp) return;
  const OpTable& op = *a.ops;
  const Gas<double> g{a.gamma, a.gm1, 2.0 * a.gm1};
  const int k = (int)(w / Nfp), f = (int)(w % Nfp);
  const int lin = a.nbr[(size_t)k * Nfp + f];
  const int kP = lin / Nfp, fP = lin % Nfp;
  auto pos = [&](int ff) { return ff < 2 * n ? 2 * (ff % n) + ff / n : 2 * n + 2 * (ff % n) + (ff / n - 2); };
  const long long key = (long long)k * Nfp + pos(f), keyP = (long long)kP * Nfp + pos(fP);
  if (key >= keyP) return;  // the partner's item (or a face without a partner)
  auto node = [&](int ff) {
    const int side = ff / n, tt = ff % n;
    return side == 0 ? n * tt : side == 1 ? (n - 1) + n * tt : side == 2 ? tt : tt + n * (n - 1);
  };
  auto lidx = [&](int kk, int ff) {  // the factor of face node ff in Lpre
    const int side = ff / n, tt = ff % n;
    const int idx = side == 0 ? (n + 1) * tt : side == 1 ? n + (n + 1) * tt : side == 2 ? tt : tt + n * n;
    return (size_t)kk * 2 * NSF + (side < 2 ? 0 : NSF) + idx;
  };
  double vA[4], vB[4];
  const double* UA = a.Uq + 4 * ((size_t)k * Nq + node(f));
  const double* UB = a.Uq + 4 * ((size_t)kP * Nq + node(fP));
  v_ufun_rn(g, UA, vA);
  v_ufun_rn(g, UB, vB);
  const int d = f < 2 * n ? 0 : 1;  // both faces lie on the same axis
  // every product rounded by itself (no FMA contraction), as the reference's psif and
  // dv .* f* are: equal states must give a jump of exactly 0
  const double dpsi = __dsub_rn(__dmul_rn(a.gm1, UA[1 + d]), __dmul_rn(a.gm1, UB[1 + d]));
  // BF / B on the axis: the x (y) component of f* at an x (y) face
  auto dvf = [&](int kk, int ff, const double* dv, const double* BF) {
    const double* G = a.geomx + (size_t)kk * kGeomStride;
    const int side = ff / n, tt = ff % n;
    const double Bf = (side == 0 || side == 2) ? -op.w1D[tt] : op.w1D[tt];
    const double B = (d == 0 ? (side < 2 ? G[1] : G[2]) : (side < 2 ? G[3] : G[4])) * Bf;
    double p[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) p[c] = __dmul_rn(dv[c], __ddiv_rn(BF[((size_t)kk * Nfp + ff) * 8 + 4 * d + c], B));
    return __dadd_rn(__dadd_rn(__dadd_rn(p[0], p[1]), p[2]), p[3]);
  };
  auto solve = [&](double Lown, double Lpar, double dvfH, double dvfL, double dps) {
    const double l = fmin(Lown, Lpar);
    auto fok = [&](double li) { return __dadd_rn(__dmul_rn(li, dvfH), __dmul_rn(1.0 - li, dvfL)) <= dps; };
    if (fok(l)) return l;
    double x_valid = 0.0, x_invalid = l;
    for (int iter = 0; iter <= 20; ++iter) {
      const double x_new = 0.5 * (x_valid + x_invalid);
      if (fok(x_new))
        x_valid = x_new;
      else
        x_invalid = x_new;
    }
    return x_valid;
  };
  double dvA[4], dvB[4];
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    dvA[c] = __dsub_rn(vA[c], vB[c]);
    dvB[c] = __dsub_rn(vB[c], vA[c]);
  }
  const size_t iA = lidx(k, f), iB = lidx(kP, fP);
  const double LA = solve(a.Lpre[iA], a.Lpre[iB], dvf(k, f, dvA, a.BFH), dvf(k, f, dvA, a.BFL), dpsi);
  const double LB = solve(a.Lpre[iB], LA, dvf(kP, fP, dvB, a.BFH), dvf(kP, fP, dvB, a.BFL), -dpsi);
  a.Lpre[iA] = LA;
  a.Lpre[iB] = LB;
}

template <int N1D>
__global__ void __launch_bounds__(256) k_es_interface(StageArgs a) {
  es_interface_body<N1D>(a, blockIdx.x * (long long)blockDim.x + threadIdx.x);
}

template <int N1D>
__global__ void __launch_bounds__(Cfg<N1D>::THREADS) k_gauss_proj(StageArgs a) {
  extern __shared__ __align__(16) double sm[];
  gauss_proj_body<N1D>(a, blockIdx.x * a.epb, sm);
}

// =====================================================================================
// Kernel A
// =====================================================================================

// Phase P6 for one high-order pair pp of an axis-aligned element: the pair's own axis only
// (fS_axis; the other half of the pair's scratch slot is not written, and not read), scaled
// by S and the element's geometry. Every layout calls this one body for such pairs.
template <int N1D, typename TH>
__device__ __forceinline__ void pair_term_aa(const OpTable& op, const Gas<double>& g, const Gas<float>& gf,
                                             double* base, int pp, bool acc64) {
  using C = Cfg<N1D>;
  const double* G = base + C::O_GEO;
  const int i = op.hp_i[pp], j = op.hp_j[pp], ax = op.hp_axis[pp];
  if (sizeof(TH) == 8) {
    const double Sa = (ax == 0 ? G[1] : G[4]) * op.hp_S[pp];
    double F[4];
    fS_axis(g, base + C::O_PRIM + 6 * i, base + C::O_PRIM + 6 * j, ax, F);
    double* out = base + C::O_SCR + 8 * pp;
#pragma unroll
    for (int c = 0; c < 4; ++c) out[4 * ax + c] = Sa * F[c];
  } else {
    const float4* Pf = reinterpret_cast<const float4*>(base + C::O_PRIM);
    const float4 qi = Pf[i], qj = Pf[j];
    const float UL[4] = {qi.x, qi.y, qi.z, qi.w};
    const float UR[4] = {qj.x, qj.y, qj.z, qj.w};
    const float* Gf = reinterpret_cast<const float*>(G + 12);
    const float sa = (ax == 0 ? Gf[0] : Gf[3]) * op.hp_Sf[pp];
    float F[4];
    fS_f32_axis(gf, UL, UR, ax, F);
    if (acc64) {
      double* outd = base + C::O_SCR + 8 * pp;
#pragma unroll
      for (int c = 0; c < 4; ++c) outd[4 * ax + c] = (double)(sa * F[c]);
    } else {
      float* outf = reinterpret_cast<float*>(base + C::O_SCR) + 8 * pp;
#pragma unroll
      for (int c = 0; c < 4; ++c) outf[4 * ax + c] = sa * F[c];
    }
  }
}

// Phase P7 for the axis-ax half of node m of an axis-aligned element (assemble_rhs!,
// flux_differencing.jl:331-361): the pair terms of the node's line in the merged gather
// order, the node's face term on that axis, lift by 1/wq and scale by 1/J. Every layout
// calls this one body for such nodes.
template <int N1D, typename TH>
__device__ __forceinline__ void node_half_aa(const OpTable& op, double* base, int m, int ax, bool acc64) {
  using C = Cfg<N1D>;
  constexpr int n = C::n;
  const int ir = m % n, is = m / n;
  const int f = ax == 0 ? (ir == 0 ? is : (ir == n - 1 ? n + is : -1))
                        : (is == 0 ? 2 * n + ir : (is == n - 1 ? 3 * n + ir : -1));
  const double* BH = base + C::O_BFH + 8 * (f < 0 ? 0 : f) + 4 * ax;
  double* R = base + C::O_RXYH + 8 * m + 4 * ax;
  if (sizeof(TH) == 8 || acc64) {
    const double rJ = base[C::O_GEO + 11];
    const double rw = op.rwq[m];
    double Q[4] = {0, 0, 0, 0};
    for (int t = 0; t < n - 1; ++t) {
      const double* sf = base + C::O_SCR + 8 * op.hga_pair[ax][m][t] + 4 * ax;
      const int sg = op.hga_sign[ax][m][t];
#pragma unroll
      for (int c = 0; c < 4; ++c) Q[c] = Q[c] + signed_by(sf[c], sg);
    }
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const double Bs = f < 0 ? 0.0 : rw * BH[c];
      R[c] = (-(rw * Q[c] + Bs)) * rJ;
    }
  } else {
    const float* sfb = reinterpret_cast<const float*>(base + C::O_SCR);
    const float rwf = op.rwqf[m];
    const float rJf = reinterpret_cast<const float*>(base + C::O_GEO + 12)[4];
    float Q[4] = {0, 0, 0, 0};
    for (int t = 0; t < n - 1; ++t) {
      const float* sf = sfb + 8 * op.hga_pair[ax][m][t] + 4 * ax;
      const int sg = op.hga_sign[ax][m][t];
#pragma unroll
      for (int c = 0; c < 4; ++c) Q[c] = Q[c] + signed_by(sf[c], sg);
    }
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const float Bs = f < 0 ? 0.0f : rwf * (float)BH[c];
      R[c] = (double)((-(rwf * Q[c] + Bs)) * rJf);
    }
  }
}

// Phases P6 and P7 of axis-aligned elements with whole lines per warp: the block's lines
// (element e, axis ax, line l) are dealt to its warps LPW at a time; a warp computes its
// lines' pairs (lane -> line, pair), synchronizes only itself, and then gathers and lifts
// its lines' node halves (lane -> line, node), since on such elements the x half of a
// node's volume term depends only on the pairs of its r-line and the y half only on its
// s-line. The arithmetic is the flat layout's (pair_term_aa, node_half_aa), so the results
// are the same bits.
template <int N1D, typename TH>
__device__ __forceinline__ void pairs_lines_per_warp(const OpTable& op, const Gas<double>& g, const Gas<float>& gf,
                                                     double* sm, int PE, int Ke, bool acc64) {
  using C = Cfg<N1D>;
  constexpr int n = C::n;
  constexpr int PPL = n * (n - 1) / 2;  // pairs per line
  // lines per warp: as many as both steps fit in 32 lanes (PPL pairs, then n nodes, per line)
  constexpr int LPW = cmin(32 / PPL, 32 / n);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int nlines = Ke * 2 * n;  // line id = (e * 2 + ax) * n + l
  for (int l0 = warp * LPW; l0 < nlines; l0 += nwarps * LPW) {
    const int lp = l0 + lane / PPL;
    if (lane < LPW * PPL && lp < nlines) {
      const int e = lp / (2 * n), ax = (lp / n) % 2, l = lp % n;
      pair_term_aa<N1D, TH>(op, g, gf, sm + e * PE, (ax * n + l) * PPL + lane % PPL, acc64);
    }
    __syncwarp();
    const int ln = l0 + lane / n;
    if (lane < LPW * n && ln < nlines) {
      const int e = ln / (2 * n), ax = (ln / n) % 2, l = ln % n, a2 = lane % n;
      node_half_aa<N1D, TH>(op, sm + e * PE, ax == 0 ? a2 + n * l : l + n * a2, ax, acc64);
    }
    __syncwarp();
  }
}
// Body of kernel A for the E elements k0 .. k0+E-1 of the solve `a`; every early return
// is uniform over the block. Used by the one-solve kernel and the batched kernel.
// EXT: compiles the branches of kExtFlags; without it those flags are masked off, so their
// tests fold away and the common modes run a lean instruction stream.
template <int N1D, typename TH, bool GAUSS = false, bool EXT = false>
__device__ __forceinline__ void stage_a_body(const StageArgs& a, int k0, double* sm) {
  using C = Cfg<N1D>;
  constexpr int n = C::n, Nq = C::Nq, Nfp = C::Nfp, NSF = C::NSF, NEV = C::NEV;
  constexpr int PE = GAUSS ? C::PER_ELEM_G : (EXT ? C::PER_ELEM_X : C::PER_ELEM_A);
  static_assert(!GAUSS || sizeof(TH) == 8, "Gauss collocation runs in FP64");
  if (a.scal[S_DONE] != 0.0) return;
  const int E = a.epb;
  int* s_list = reinterpret_cast<int*>(sm + PE * E);  // [0]: count, then eval indices
  const OpTable& op = *a.ops;
  const int tid = threadIdx.x, bs = blockDim.x;
  const int Ke = min(E, a.K - k0);
  if (Ke <= 0) return;
  static_assert(!GAUSS || EXT, "Gauss collocation is an EXT mode");
  const int flags = EXT ? a.flags : (a.flags & ~kExtFlags);
  const bool aa = flags & F_AXIS_ALIGNED;
  Gas<double> g{a.gamma, a.gm1, 2.0 * a.gm1};
  const double dt_lim = a.scal[S_DT_LIM];
  const double t_now = a.scal[S_T];

  // ---- P0: geometry and state. The geometry factors (geom_factor) come from the
  //      solve's per-element table when it has one (made once at set-up), else one item
  //      per (element, factor)
  if (a.geomx) {
    for (int w = tid; w < Ke * kGeomStride; w += bs) {
      const int e = w / kGeomStride, q = w % kGeomStride;
      sm[e * PE + C::O_GEO + q] = a.geomx[(size_t)k0 * kGeomStride + w];
    }
  } else {
    constexpr int NG = sizeof(TH) == 4 ? kGeomFactors : 12;
    for (int w = tid; w < Ke * NG; w += bs) {
      const int e = w / NG, q = w % NG;
      geom_factor(a.geom + 5 * (size_t)(k0 + e), q, sm + e * PE + C::O_GEO);
    }
  }
  if (tid == 0) {
    s_list[0] = 0;
    s_list[NEV * E + 1] = 0;  // the count of the bisections' list (P9)
  }
  for (int w = tid; w < Ke * Nq * 4; w += bs) {
    int e = w / (Nq * 4), r = w % (Nq * 4);
    sm[e * PE + C::O_U + r] = a.Uq[(size_t)k0 * Nq * 4 + w];
  }
  if (GAUSS) {  // the projected face states and theta of this stage (face projection kernel)
    for (int w = tid; w < Ke * Nfp * 4; w += bs) {
      int e = w / (Nfp * 4), r = w % (Nfp * 4);
      sm[e * PE + C::O_UF + r] = a.ufproj[(size_t)k0 * Nfp * 4 + w];
    }
    for (int w = tid; w < Ke * Nfp; w += bs) {
      int e = w / Nfp, f = w % Nfp;
      sm[e * PE + C::O_TH + f] = a.theta[((size_t)(a.nstage - 1) * a.K + k0 + e) * Nfp + f];
    }
  }
  __syncthreads();

  // ---- P1: per-node primitives, fluxes, wavespeeds along the r- and s-normals
  const bool do_low = flags & F_DO_LOW, do_high = flags & F_DO_HIGH;
  for (int w = tid; w < Ke * Nq; w += bs) {
    int e = w / Nq, m = w % Nq;
    double* base = sm + e * PE;
    const double* G = base + C::O_GEO;
    const double* U = base + C::O_U + 4 * m;
    if (flags & F_KPP) {  // fluxes (sin u, cos u) (KPP.jl:13-18), wavespeed 1, indicator u
      double* F = base + C::O_FLUX + 8 * m;
#pragma unroll
      for (int c = 0; c < 8; ++c) F[c] = 0.0;
      F[0] = sin(U[0]);
      F[4] = cos(U[0]);
      base[C::O_WS + 2 * m] = 1.0;
      base[C::O_WS + 2 * m + 1] = 1.0;
      if (flags & F_SHOCK) base[C::O_LAMI + m] = U[0];
      base[C::O_PRIM + 6 * m] = U[0];
      continue;
    }
    double rho = U[0], rhou = U[1], rhov = U[2], E = U[3];
    double rr = rcp(rho);
    double p = g.gm1 * fma(-0.5, (rhou * rhou + rhov * rhov) * rr, E);
    // a state the reference would stop on (DomainError from log or sqrt of a negative,
    // flux_differencing.jl:49-50): density or pressure -0, negative or NaN, by their bits
    if (__double_as_longlong(rho) <= 0 || __double_as_longlong(rho) > 0x7ff0000000000000LL ||
        __double_as_longlong(p) <= 0 || __double_as_longlong(p) > 0x7ff0000000000000LL)
      atomicOr(a.status, ST_NOT_POSITIVE);
    double u = rhou * rr, v = rhov * rr;
    double* F = base + C::O_FLUX + 8 * m;
    double Ep = E + p;
    F[0] = rhou;
    F[1] = rhou * u + p;
    F[2] = rho * u * v;
    F[3] = u * Ep;
    F[4] = rhov;
    F[5] = F[2];
    F[6] = rhov * v + p;
    F[7] = v * Ep;
    double* Ws = base + C::O_WS + 2 * m;
    if (aa) {
      // the unit normals are (+-1, 0) and (0, +-1) exactly (g/sqrt(g^2) = +-1), so the
      // normal momentum is +-rhou or +-rhov, and its sign does not enter the wavespeed
      Ws[0] = wavespeed_r(g, rr, rhou, E);
      Ws[1] = wavespeed_r(g, rr, rhov, E);
    } else {
      Ws[0] = wavespeed_r(g, rr, G[6] * rhou + G[7] * rhov, E);
      Ws[1] = wavespeed_r(g, rr, G[9] * rhou + G[10] * rhov, E);
    }
    if (flags & (F_SHOCK | F_RELAXED)) base[C::O_LAMI + m] = rho * p;  // the indicator rho p (shock_capture.jl:92-103)
    if (do_high) {
      if (sizeof(TH) == 8) {
        double* Pm = base + C::O_PRIM + 6 * m;
        double beta = rho * rcp(2.0 * p);
        Pm[0] = rho;
        Pm[1] = u;
        Pm[2] = v;
        Pm[3] = beta;
        Pm[4] = log_fast(rho, op);
        Pm[5] = log_fast(beta, op);
      } else {
        // FP32 (rho, u, v, beta) per node, converted once here rather than per pair
        float rf = (float)rho;
        reinterpret_cast<float4*>(base + C::O_PRIM)[m] = make_float4(rf, (float)u, (float)v, rf / (2.0f * (float)p));
      }
    }
  }
  if (GAUSS) {
    // primitives of the projected face states (calculate_primitive_variables!, :39-52)
    for (int w = tid; w < Ke * Nfp; w += bs) {
      int e = w / Nfp, f = w % Nfp;
      double* base = sm + e * PE;
      const double* U = base + C::O_UF + 4 * f;
      const double rr = rcp(U[0]);
      const double p = g.gm1 * fma(-0.5, (U[1] * U[1] + U[2] * U[2]) * rr, U[3]);
      const double beta = U[0] * rcp(2.0 * p);
      double* Pm = base + C::O_PF + 6 * f;
      Pm[0] = U[0];
      Pm[1] = U[1] * rr;
      Pm[2] = U[2] * rr;
      Pm[3] = beta;
      Pm[4] = log_fast(U[0], op);
      Pm[5] = log_fast(beta, op);
    }
    // is_Vf_limited (flux_differencing.jl:316-318): any theta < 1 on the element, into O_XT + 1
    for (int e = tid; e < Ke; e += bs) {
      double* base = sm + e * PE;
      double lim = 0.0;
      for (int f = 0; f < Nfp; ++f)
        if (base[C::O_TH + f] < 1.0) lim = 1.0;
      base[C::O_XT + 1] = lim;
    }
  }
  __syncthreads();

  // ---- P1b: smoothness indicator (shock_capture.jl:49-81): modal energies of the
  //      indicator through inv(VDM), smoothness max(E_N, E_{N-1}) / E. Hennemann
  //      blending factor max(min(1 - alpha, 1), 1/2) (:118-137) into G[15]; the relaxed
  //      bounds' smoothness factor (update_smoothness_factor!, subcell.jl:937-956) into O_XT
  if (flags & (F_SHOCK | F_RELAXED)) {
    for (int w = tid; w < Ke * Nq; w += bs) {
      const int e = w / Nq, i = w % Nq;
      double* base = sm + e * PE;
      const double* Vi = op.VDMinv + i * Nq;
      double sum = 0.0;
      for (int j = 0; j < Nq; ++j) sum = fma(Vi[j], base[C::O_LAMI + j], sum);
      base[C::O_SCR + i] = sum * sum;
    }
    __syncthreads();
    for (int e = tid; e < Ke; e += bs) {
      double* base = sm + e * PE;
      double modeN = 0.0, modeNm1 = 0.0, total = 0.0;
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
          const double energy = base[C::O_SCR + i + n * j];
          if (i == n - 1 || j == n - 1) modeN += energy;
          if (i == n - 2 || j == n - 2) modeNm1 += energy;
          total += energy;
        }
      const double smooth = fmax(modeN / total, modeNm1 / total);
      if (flags & F_SHOCK) {
        const double alpha = 1.0 / (1.0 + exp(a.sc_q * (smooth - a.sc_TN)));
        base[C::O_GEO + 15] = fmax(fmin(1.0 - alpha, 1.0), 0.5);
      }
      if (flags & F_RELAXED) {
        // kappa = 1; log(10, x) = log(x) / log(10), log(10) as the correctly rounded
        // constant (a device log(10.0) may be folded at compile time in one translation
        // unit and evaluated in another, which would give batch members other bits)
        const double sk = log(smooth) / 2.302585092994046;
        double eps;
        if (sk < a.s0 - 1.0)
          eps = 0.0;
        else if (sk > a.s0 + 1.0)
          eps = 1.0;
        else
          eps = 0.5 - 0.5 * sin(3.141592653589793 * (sk - a.s0) / 2.0);
        base[C::O_XT] = eps;
      }
    }
    __syncthreads();
  }

  // ---- P2: low-order volume pairs (accumulate_low_order_rhs_volume!, :139-173)
  if (do_low) {
    for (int w = tid; w < Ke * C::NPL; w += bs) {
      int e = w / C::NPL, pp = w % C::NPL;
      double* base = sm + e * PE;
      const double* G = base + C::O_GEO;
      int i = op.lp_i[pp], j = op.lp_j[pp], ax = op.lp_axis[pp];
      double S = op.lp_S[pp];
      double g1 = ax == 0 ? G[1] : G[2], g2 = ax == 0 ? G[3] : G[4], gn = ax == 0 ? G[5] : G[8];
      double S0x = g1 * S, S0y = g2 * S;
      double nn = fabs(S) * gn;
      double wsi = base[C::O_WS + 2 * i + ax], wsj = base[C::O_WS + 2 * j + ax];
      double lam = nn * fmax(wsi, wsj);
      const double* Ui = base + C::O_U + 4 * i;
      const double* Uj = base + C::O_U + 4 * j;
      const double* Fi = base + C::O_FLUX + 8 * i;
      const double* Fj = base + C::O_FLUX + 8 * j;
      double* out = base + C::O_SCR + 9 * pp;
      bool visc_x = fabs(S0x) > 1e-10;
      // 2 S0 * (fi + fj)/2 is S0 * (fi + fj) exactly (power-of-two factors)
      if (aa) {
        // the pair's terms on the other axis are zero; one instruction stream for both axes
        const int o = 4 * ax;
        const double S0 = ax == 0 ? S0x : S0y;
        const bool vis_on = ax == 0 ? visc_x : !visc_x;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          double vis = vis_on ? lam * (Uj[c] - Ui[c]) : 0.0;
          out[o + c] = fma(S0, Fi[o + c] + Fj[o + c], -vis);
        }
      } else {
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          double vis = visc_x ? lam * (Uj[c] - Ui[c]) : 0.0;
          out[c] = fma(S0x, Fi[c] + Fj[c], -vis);
        }
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          double vis = visc_x ? 0.0 : lam * (Uj[c] - Ui[c]);
          out[4 + c] = fma(S0y, Fi[4 + c] + Fj[4 + c], -vis);
        }
      }
      out[8] = lam;
    }
    __syncthreads();
    // ---- P3: gather Q0F1 in the order of the nnz loop; rhsxyL = 0 - Q0F1
    for (int w = tid; w < Ke * Nq; w += bs) {
      int e = w / Nq, m = w % Nq;
      double* base = sm + e * PE;
      double Q[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      double lam = 0.0;
      int cnt = op.lg_count[m];
      if (aa) {
        // r-line pairs feed the x half, s-line pairs the y half, each in the merged order
#pragma unroll
        for (int ax = 0; ax < 2; ++ax) {
          const int ca = op.lga_count[ax][m];
          for (int t = 0; t < ca; ++t) {
            const double* sf = base + C::O_SCR + 9 * op.lga_pair[ax][m][t];
            const int sg = op.lga_sign[ax][m][t];
#pragma unroll
            for (int c = 0; c < 4; ++c) Q[4 * ax + c] = Q[4 * ax + c] + signed_by(sf[4 * ax + c], sg);
          }
        }
        for (int t = 0; t < cnt; ++t) lam += base[C::O_SCR + 9 * op.lg_pair[m][t] + 8];
      } else {
        for (int t = 0; t < cnt; ++t) {
          int pp = op.lg_pair[m][t];
          const double* sf = base + C::O_SCR + 9 * pp;
          const int sg = op.lg_sign[m][t];
#pragma unroll
          for (int c = 0; c < 8; ++c) Q[c] = Q[c] + signed_by(sf[c], sg);
          lam += sf[8];
        }
      }
      double* R = base + C::O_RXYL + 8 * m;
#pragma unroll
      for (int c = 0; c < 8; ++c) R[c] = -Q[c];
      base[C::O_LAMI + m] = lam;
    }
  }
  __syncthreads();

  // ---- P4: surface terms, shared by the low-order (:175-204) and high-order
  //          (flux_differencing.jl:90-151, 223-272) paths
  for (int w = tid; w < Ke * Nfp; w += bs) {
    int e = w / Nfp, f = w % Nfp;
    const int k = k0 + e;
    double* base = sm + e * PE;
    const double* G = base + C::O_GEO;
    int side = f / n, tt = f % n;
    int q = side == 0 ? n * tt : side == 1 ? (n - 1) + n * tt : side == 2 ? tt : tt + n * (n - 1);
    double wt = op.w1D[tt];
    double Bf = (side == 0 || side == 2) ? -wt : wt;
    bool xs = side < 2;
    double g1 = xs ? G[1] : G[2], g2 = xs ? G[3] : G[4], gn = xs ? G[5] : G[8];
    double nh1 = xs ? G[6] : G[9], nh2 = xs ? G[7] : G[10];
    double B1 = g1 * Bf, B2 = g2 * Bf;
    double nn = wt * gn;
    double n1 = Bf < 0 ? -nh1 : nh1, n2 = Bf < 0 ? -nh2 : nh2;
    // the face values of the low-order flux: the node's (LaxFriedrichsOnNodalVal) or, with
    // LaxFriedrichsOnProjectedVal on Gauss nodes, the projected face state (update_face_values!,
    // low_order_graph_viscosity.jl:51-71), the neighbour's from ufproj
    const bool projL = GAUSS && (flags & F_LFPROJ);
    const double* Uf = projL ? base + C::O_UF + 4 * f : base + C::O_U + 4 * q;
    double ws_own = projL ? wavespeed_r(g, rcp(Uf[0]), n1 * Uf[1] + n2 * Uf[2], Uf[3])
                          : base[C::O_WS + 2 * q + (xs ? 0 : 1)];
    size_t fk = (size_t)k * Nfp + f;
    int lin = a.nbr[fk];
    bool self = lin == (int)fk;
    double Unb[4];
    if (self) {
#pragma unroll
      for (int c = 0; c < 4; ++c) Unb[c] = Uf[c];
    } else if (projL) {
#pragma unroll
      for (int c = 0; c < 4; ++c) Unb[c] = __ldg(a.ufproj + 4 * (size_t)lin + c);
    } else {
      int kP = lin / Nfp, iP = lin % Nfp;
      int sP = iP / n, tP = iP % n;
      int qP = sP == 0 ? n * tP : sP == 1 ? (n - 1) + n * tP : sP == 2 ? tP : tP + n * (n - 1);
      if (kP >= k0 && kP < k0 + Ke) {
        const double* src = sm + (kP - k0) * PE + C::O_U + 4 * qP;
#pragma unroll
        for (int c = 0; c < 4; ++c) Unb[c] = src[c];
      } else {
        const double* src = a.Uq + ((size_t)kP * Nq + qP) * 4;
#pragma unroll
        for (int c = 0; c < 4; ++c) Unb[c] = __ldg(src + c);
      }
    }
    int code = a.bc[fk];
    double uP[4];
    if (code == BC_INTERIOR) {
#pragma unroll
      for (int c = 0; c < 4; ++c) uP[c] = Unb[c];
    } else if (code == BC_INFLOW) {
      const double* iv = a.Ival + 4 * (size_t)a.bcidx[fk];
#pragma unroll
      for (int c = 0; c < 4; ++c) uP[c] = iv[c];
    } else if (code == BC_OUTFLOW) {  // the own node's Uq (get_uP_and_enforce_BC!, :117-123)
      const double* Uq = base + C::O_U + 4 * q;
#pragma unroll
      for (int c = 0; c < 4; ++c) uP[c] = Uq[c];
    } else if (code == BC_WALL) {
      double mn = Uf[1] * n1 + Uf[2] * n2;
      uP[0] = Uf[0];
      uP[1] = Uf[1] - 2.0 * mn * n1;
      uP[2] = Uf[2] - 2.0 * mn * n2;
      uP[3] = Uf[3];
    } else {
      const double* xy = a.xyS + 2 * (size_t)a.bcidx[fk];
      bool post = xy[0] < a.shock_x0 + (xy[1] + a.shock_speed * t_now) * a.shock_inv_slope;
#pragma unroll
      for (int c = 0; c < 4; ++c) uP[c] = post ? a.shock_post[c] : a.shock_pre[c];
    }
    const bool kpp = flags & F_KPP;
    double rrP = kpp ? 0.0 : rcp(uP[0]);
    double wsP = ws_own;
    if (!self && !kpp) {
      double rrN = (code == BC_INTERIOR) ? rrP : rcp(Unb[0]);
      wsP = wavespeed_r(g, rrN, aa ? (xs ? Unb[1] : Unb[2]) : n1 * Unb[1] + n2 * Unb[2], Unb[3]);
    }
    double lamB = 0.5 * nn * fmax(ws_own, wsP);
    double Fp[8];  // the projected face state's fluxes (projL)
    if (projL) fluxes_r(g, Uf, rcp(Uf[0]), Fp, Fp + 4);
    const double* Ff = projL ? Fp : base + C::O_FLUX + 8 * q;
    double* BL = base + C::O_BFL + 8 * f;
    double* BH = base + C::O_BFH + 8 * f;
    bool lf_zero_high = (code == BC_INFLOW || code == BC_OUTFLOW || code == BC_SHOCK);
    // B * (f(U) + f(uP))/2 with the exact factor 1/2 taken into B
    const double hB1 = 0.5 * B1, hB2 = 0.5 * B2;
    if (aa) {
      // sxJ = ryJ = 0: the face's terms have only its own axis' half; the other is zero
      double fP[4];
      if (kpp) {
        fP[0] = xs ? sin(uP[0]) : cos(uP[0]);
        fP[1] = fP[2] = fP[3] = 0.0;
      } else {
        flux_axis_r(g, uP, rrP, xs, fP);
      }
      const double hB = xs ? hB1 : hB2;
      const int o = xs ? 0 : 4;
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        double lf = lamB * (uP[c] - Uf[c]);
        double b = hB * (Ff[o + c] + fP[c]);
        double bl = b - lf;
        BL[o + c] = bl;
        BL[4 - o + c] = 0.0;
        BH[o + c] = lf_zero_high ? b : bl;
        BH[4 - o + c] = 0.0;
      }
    } else {
      double fPx[4], fPy[4];
      if (kpp) {
        fPx[0] = sin(uP[0]);
        fPy[0] = cos(uP[0]);
        fPx[1] = fPx[2] = fPx[3] = fPy[1] = fPy[2] = fPy[3] = 0.0;
      } else {
        fluxes_r(g, uP, rrP, fPx, fPy);
      }
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        double lf = lamB * (uP[c] - Uf[c]);
        double bx = hB1 * (Ff[c] + fPx[c]), by = hB2 * (Ff[4 + c] + fPy[c]);
        BL[c] = xs ? bx - lf : bx;
        BL[4 + c] = xs ? by : by - lf;
        if (lf_zero_high) {
          BH[c] = bx;
          BH[4 + c] = by;
        } else {
          BH[c] = BL[c];
          BH[4 + c] = BL[4 + c];
        }
      }
    }
    // the face's CFL term: lambda_B_CFL (low_order_graph_viscosity.jl:301-309): lambdaB, or
    // with the projected-value flux alpha lambdaB + |B| ws / 2 (alpha = 1 for KPP, else
    // find_alpha of the face values, which are the nodal values on LGL nodes)
    double lam_cfl = lamB;
    if ((flags & F_LFPROJ) && (flags & F_CFL))
      lam_cfl = (kpp ? 1.0 : find_alpha(base + C::O_U + 4 * q, Uf, a.POSTOL)) * lamB + 0.5 * nn * ws_own;
    base[C::O_LAMB + f] = lam_cfl;
  }
  __syncthreads();
  if (GAUSS && do_high) {
    // ---- P4g: the high-order surface flux on the projected face states
    //      (calculate_interface_dissipation_coeff!, enforce_BC!, flux_differencing.jl:90-151;
    //      accumulate_numerical_flux! with LaxFriedrichsOnProjectedVal, :223-272): the
    //      neighbour's projected state across the face; outflow takes the own node's Uq,
    //      walls reflect the own projected state; LF coefficient from both wavespeeds
    for (int w = tid; w < Ke * Nfp; w += bs) {
      int e = w / Nfp, f = w % Nfp;
      const int k = k0 + e;
      double* base = sm + e * PE;
      const double* G = base + C::O_GEO;
      int side = f / n, tt = f % n;
      int q = side == 0 ? n * tt : side == 1 ? (n - 1) + n * tt : side == 2 ? tt : tt + n * (n - 1);
      double wt = op.w1D[tt];
      double Bf = (side == 0 || side == 2) ? -wt : wt;
      bool xs = side < 2;
      double g1 = xs ? G[1] : G[2], g2 = xs ? G[3] : G[4], gn = xs ? G[5] : G[8];
      double nh1 = xs ? G[6] : G[9], nh2 = xs ? G[7] : G[10];
      double B1 = g1 * Bf, B2 = g2 * Bf;
      double nn = wt * gn;
      double n1 = Bf < 0 ? -nh1 : nh1, n2 = Bf < 0 ? -nh2 : nh2;
      const double* uf = base + C::O_UF + 4 * f;
      size_t fk = (size_t)k * Nfp + f;
      int lin = a.nbr[fk];
      bool self = lin == (int)fk;
      double ufn[4];
#pragma unroll
      for (int c = 0; c < 4; ++c) ufn[c] = self ? uf[c] : __ldg(a.ufproj + 4 * (size_t)lin + c);
      int code = a.bc[fk];
      double uP[4];
      if (code == BC_INTERIOR) {
#pragma unroll
        for (int c = 0; c < 4; ++c) uP[c] = ufn[c];
      } else if (code == BC_INFLOW) {
        const double* iv = a.Ival + 4 * (size_t)a.bcidx[fk];
#pragma unroll
        for (int c = 0; c < 4; ++c) uP[c] = iv[c];
      } else if (code == BC_OUTFLOW) {
        const double* Uq = base + C::O_U + 4 * q;
#pragma unroll
        for (int c = 0; c < 4; ++c) uP[c] = Uq[c];
      } else if (code == BC_WALL) {
        double mn = uf[1] * n1 + uf[2] * n2;
        uP[0] = uf[0];
        uP[1] = uf[1] - 2.0 * mn * n1;
        uP[2] = uf[2] - 2.0 * mn * n2;
        uP[3] = uf[3];
      } else {
        const double* xy = a.xyS + 2 * (size_t)a.bcidx[fk];
        bool post = xy[0] < a.shock_x0 + (xy[1] + a.shock_speed * t_now) * a.shock_inv_slope;
#pragma unroll
        for (int c = 0; c < 4; ++c) uP[c] = post ? a.shock_post[c] : a.shock_pre[c];
      }
      const double rrf = rcp(uf[0]);
      const double lam = wavespeed_r(g, rrf, n1 * uf[1] + n2 * uf[2], uf[3]);
      const double lamN = self ? lam : wavespeed_r(g, rcp(ufn[0]), n1 * ufn[1] + n2 * ufn[2], ufn[3]);
      double LFc = 0.5 * nn * fmax(lam, lamN);
      if (code == BC_INFLOW || code == BC_OUTFLOW || code == BC_SHOCK) LFc = 0.0;
      double ffx[4], ffy[4], fPx[4], fPy[4];
      fluxes_r(g, uf, rrf, ffx, ffy);
      fluxes_r(g, uP, rcp(uP[0]), fPx, fPy);
      const double hB1 = 0.5 * B1, hB2 = 0.5 * B2;
      double* BH = base + C::O_BFH + 8 * f;
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const double lf = LFc * (uP[c] - uf[c]);
        const double bx = (aa && !xs) ? 0.0 : hB1 * (ffx[c] + fPx[c]);
        const double by = (aa && xs) ? 0.0 : hB2 * (ffy[c] + fPy[c]);
        BH[c] = xs ? bx - lf : bx;
        BH[4 + c] = xs ? by : by - lf;
      }
    }
    __syncthreads();
  }

  // ---- P5: finish the low-order RHS, scale by mass, positivity CFL
  double dt_loc = __longlong_as_double(0x7ff0000000000000LL);
  bool nan_seen = false;
  if (do_low) {
    for (int w = tid; w < Ke * Nq; w += bs) {
      int e = w / Nq, m = w % Nq;
      double* base = sm + e * PE;
      int ir = m % n, is = m / n;
      int fl[2], nf = 0;
      if (ir == 0) fl[nf++] = is;
      if (ir == n - 1) fl[nf++] = n + is;
      if (is == 0) fl[nf++] = 2 * n + ir;
      if (is == n - 1) fl[nf++] = 3 * n + ir;
      double* R = base + C::O_RXYL + 8 * m;
      double lam = base[C::O_LAMI + m];
      if (aa) {
        // at most one x face (its x half) and one y face (its y half); absent ones add 0
        const int fx = ir == 0 ? is : (ir == n - 1 ? n + is : -1);
        const int fy = is == 0 ? 2 * n + ir : (is == n - 1 ? 3 * n + ir : -1);
        const double* BLx = base + C::O_BFL + 8 * (fx < 0 ? 0 : fx);
        const double* BLy = base + C::O_BFL + 8 * (fy < 0 ? 0 : fy);
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          R[c] = R[c] - (fx < 0 ? 0.0 : BLx[c]);
          R[4 + c] = R[4 + c] - (fy < 0 ? 0.0 : BLy[4 + c]);
        }
        lam = lam + (fx < 0 ? 0.0 : base[C::O_LAMB + (fx < 0 ? 0 : fx)]);
        lam = lam + (fy < 0 ? 0.0 : base[C::O_LAMB + (fy < 0 ? 0 : fy)]);
      } else {
        for (int t = 0; t < nf; ++t) {
          const double* BL = base + C::O_BFL + 8 * fl[t];
#pragma unroll
          for (int c = 0; c < 8; ++c) R[c] = R[c] - BL[c];
          lam += base[C::O_LAMB + fl[t]];
        }
      }
      double wJ = base[C::O_GEO] * op.wq[m];
      double rwJ = base[C::O_GEO + 11] * op.rwq[m];  // (1/J)(1/wq)
      // wJ and 1/wJ for the limiter (the wavespeeds are no longer needed)
      base[C::O_WS + 2 * m] = wJ;
      base[C::O_WS + 2 * m + 1] = rwJ;
#pragma unroll
      for (int c = 0; c < 8; ++c) R[c] = R[c] * rwJ;
      double* rl = base + C::O_RHSL + 4 * m;
#pragma unroll
      for (int c = 0; c < 4; ++c) rl[c] = R[c] + R[4 + c];
      if (flags & F_CFL) {
        double d = a.CFL * 0.5 * wJ * rcp(lam);
        if (isnan(d)) nan_seen = true;
        dt_loc = fmin(dt_loc, d);
      }
    }
  }
  if (flags & F_CFL) {
    // block min of the CFL candidates
    for (int o = 16; o > 0; o >>= 1) dt_loc = fmin(dt_loc, __shfl_xor_sync(0xffffffffu, dt_loc, o));
    if ((tid & 31) == 0) {
      if (dt_loc > 0.0) atomicMin(a.dtmin_bits, (unsigned long long)__double_as_longlong(dt_loc));
      else if (dt_loc <= 0.0) atomicOr(a.status, ST_BAD_DT);
    }
    if (nan_seen) atomicOr(a.status, ST_NAN);
  }
  __syncthreads();
  if (flags & F_LOW_ONLY) {
    // the low-order densities for the TVD bounds of the next launch (subcell.jl:112-125)
    for (int w = tid; w < Ke * Nq; w += bs) {
      int e = w / Nq, m = w % Nq;
      const double* base = sm + e * PE;
      a.rhoL[(size_t)(k0 + e) * Nq + m] = low_update(base[C::O_U + 4 * m], dt_lim, base[C::O_RHSL + 4 * m]);
    }
    return;
  }

  // ---- P6: high-order volume pairs (flux_differencing_volume!, :164-211)
  // FP32 kernel with FP64 accumulation of the pair terms
  const bool acc64 = sizeof(TH) == 4 && (flags & F_ACC64);
  const Gas<float> gf{(float)a.gamma, (float)a.gm1, (float)(2.0 * a.gm1)};
  // whole lines per warp (a.layout 1) for axis-aligned LGL elements; the flat (element,
  // pair) and (element, node) loops otherwise. Both give the same bits.
  const bool lpw = !GAUSS && aa && !(flags & F_KPP) && a.layout == 1;
  if (do_high && lpw) {
    pairs_lines_per_warp<N1D, TH>(op, g, gf, sm, PE, Ke, acc64);
  } else if (do_high) {
    for (int w = tid; w < Ke * C::NPH; w += bs) {
      int e = w / C::NPH, pp = w % C::NPH;
      double* base = sm + e * PE;
      if (aa && !(flags & F_KPP)) {
        pair_term_aa<N1D, TH>(op, g, gf, base, pp, acc64);
        continue;
      }
      const double* G = base + C::O_GEO;
      int i = op.hp_i[pp], j = op.hp_j[pp], ax = op.hp_axis[pp];
      double S = op.hp_S[pp];
      double Sxx = (ax == 0 ? G[1] : G[2]) * S, Sxy = (ax == 0 ? G[3] : G[4]) * S;
      double* out = base + C::O_SCR + 8 * pp;
      if (sizeof(TH) == 8) {
        double Fx[4], Fy[4];
        if (flags & F_KPP)
          fS_kpp(base[C::O_PRIM + 6 * i], base[C::O_PRIM + 6 * j], Fx, Fy);
        else
          fS_fast(g, base + C::O_PRIM + 6 * i, base + C::O_PRIM + 6 * j, Fx, Fy);
        if (!aa || ax == 0) {
#pragma unroll
          for (int c = 0; c < 4; ++c) out[c] = Sxx * Fx[c];
        }
        if (!aa || ax == 1) {
#pragma unroll
          for (int c = 0; c < 4; ++c) out[4 + c] = Sxy * Fy[c];
        }
      } else {
        const float4* Pf = reinterpret_cast<const float4*>(base + C::O_PRIM);
        const float4 qi = Pf[i], qj = Pf[j];
        const float UL[4] = {qi.x, qi.y, qi.z, qi.w};
        const float UR[4] = {qj.x, qj.y, qj.z, qj.w};
        const float* Gf = reinterpret_cast<const float*>(G + 12);
        const float Sf = op.hp_Sf[pp];
        const float sx = (ax == 0 ? Gf[0] : Gf[1]) * Sf, sy = (ax == 0 ? Gf[2] : Gf[3]) * Sf;
        float Fx[4], Fy[4];
        fS_f32(gf, UL, UR, Fx, Fy);
        if (acc64) {  // the FP32 terms stored as FP64 for an exactly cancelling FP64 gather
          double* outd = base + C::O_SCR + 8 * pp;
          if (!aa || ax == 0) {
#pragma unroll
            for (int c = 0; c < 4; ++c) outd[c] = (double)(sx * Fx[c]);
          }
          if (!aa || ax == 1) {
#pragma unroll
            for (int c = 0; c < 4; ++c) outd[4 + c] = (double)(sy * Fy[c]);
          }
        } else {
          float* outf = reinterpret_cast<float*>(base + C::O_SCR) + 8 * pp;
          if (!aa || ax == 0) {
#pragma unroll
            for (int c = 0; c < 4; ++c) outf[c] = sx * Fx[c];
          }
          if (!aa || ax == 1) {
#pragma unroll
            for (int c = 0; c < 4; ++c) outf[4 + c] = sy * Fy[c];
          }
        }
      }
    }
    if (GAUSS) {
      // ---- P6g: the volume-face pairs (Nq + f, j) of Srsh_db, -B Ef (init.jl:152-155):
      //      S = -(B_f Vf[f, j]) on the face's axis, fS(projected face state, node j)
      for (int w = tid; w < Ke * Nfp * n; w += bs) {
        int e = w / (Nfp * n), r = w % (Nfp * n);
        int f = r / n, ai = r % n;
        double* base = sm + e * PE;
        const double* G = base + C::O_GEO;
        const int side = f / n, tt = f % n;
        const int j = side < 2 ? ai + n * tt : tt + n * ai;
        const double ell = (side % 2 == 0) ? op.ellm[ai] : op.ellp[ai];
        const double wt = op.w1D[tt];
        const double Bf = (side == 0 || side == 2) ? -wt : wt;
        const double Sv = -(Bf * ell);  // Srh_db (r faces) or Ssh_db (s faces); the other is 0
        const bool xs = side < 2;
        const double Sxx = (xs ? G[1] : G[2]) * Sv, Sxy = (xs ? G[3] : G[4]) * Sv;
        double* out = base + C::O_FPT + 8 * r;
        double Fx[4], Fy[4];
        fS_fast(g, base + C::O_PF + 6 * f, base + C::O_PRIM + 6 * j, Fx, Fy);
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          out[c] = (aa && !xs) ? 0.0 : Sxx * Fx[c];
          out[4 + c] = (aa && xs) ? 0.0 : Sxy * Fy[c];
        }
      }
    }
    __syncthreads();
    if (GAUSS) {
      // face rows of QF1: the pair terms of each face node in the nnz order (j ascending)
      for (int w = tid; w < Ke * Nfp * 8; w += bs) {
        int e = w / (Nfp * 8), r = w % (Nfp * 8);
        int f = r / 8, c = r % 8;
        double* base = sm + e * PE;
        const double* T = base + C::O_FPT + 8 * n * f;
        double q = 0.0;
        for (int ai = 0; ai < n; ++ai) q = q + T[8 * ai + c];
        base[C::O_QFF + 8 * f + c] = q;
      }
      __syncthreads();
      // ---- P7g: QF1 of the volume nodes (volume pairs in the gather order, then minus the
      //      face pair terms, faces ascending), lift with M \ Vh' = [1/wq, Vf'/wq] or, on an
      //      element with theta < 1, (1/wq) [I, Vf_new'] with Vf_new = theta Vf + (1 - theta)
      //      Vf_low (project_flux_difference_to_quad!, :274-314), assemble (:331-361)
      for (int w = tid; w < Ke * Nq; w += bs) {
        int e = w / Nq, m = w % Nq;
        double* base = sm + e * PE;
        int ir = m % n, is = m / n;
        const double rJ = base[C::O_GEO + 11];
        const double rw = op.rwq[m];
        const bool limited = base[C::O_XT + 1] != 0.0;
        double Q[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        if (aa) {
#pragma unroll
          for (int ax = 0; ax < 2; ++ax)
            for (int t = 0; t < n - 1; ++t) {
              const double* sf = base + C::O_SCR + 8 * op.hga_pair[ax][m][t];
              const int sg = op.hga_sign[ax][m][t];
#pragma unroll
              for (int c = 0; c < 4; ++c) Q[4 * ax + c] = Q[4 * ax + c] + signed_by(sf[4 * ax + c], sg);
            }
        } else {
          const int cnt = op.hg_count[m];
          for (int t = 0; t < cnt; ++t) {
            const double* sf = base + C::O_SCR + 8 * op.hg_pair[m][t];
            const int sg = op.hg_sign[m][t];
#pragma unroll
            for (int c = 0; c < 8; ++c) Q[c] = Q[c] + signed_by(sf[c], sg);
          }
        }
        const int fl[4] = {is, n + is, 2 * n + ir, 3 * n + ir};
        const int pos[4] = {ir, ir, is, is};  // the node's place on each face's line
        double mf[4];
#pragma unroll
        for (int t = 0; t < 4; ++t) {
          const int f = fl[t];
          const double* T = base + C::O_FPT + 8 * (n * f + pos[t]);
#pragma unroll
          for (int c = 0; c < 8; ++c) Q[c] = Q[c] - T[c];
          const double ell = (t % 2 == 0) ? op.ellm[pos[t]] : op.ellp[pos[t]];
          if (limited) {
            const double th = base[C::O_TH + f];
            const double low = pos[t] == ((t % 2 == 0) ? 0 : n - 1) ? 1.0 : 0.0;
            mf[t] = rw * (th * ell + (1 - th) * low);
          } else {
            mf[t] = op.liftf[m][t];
          }
        }
        double* R = base + C::O_RXYH + 8 * m;
#pragma unroll
        for (int c = 0; c < 8; ++c) {
          double av = rw * Q[c], bv = 0.0;
#pragma unroll
          for (int t = 0; t < 4; ++t) {
            av = av + mf[t] * base[C::O_QFF + 8 * fl[t] + c];
            bv = bv + mf[t] * base[C::O_BFH + 8 * fl[t] + c];
          }
          R[c] = (-(av + bv)) * rJ;
        }
      }
    } else {
    // ---- P7: gather QF1, lift and assemble (assemble_rhs!, :331-361)
    for (int w = tid; w < Ke * Nq; w += bs) {
      int e = w / Nq, m = w % Nq;
      double* base = sm + e * PE;
      int ir = m % n, is = m / n;
      int fl[2], nf = 0;
      if (ir == 0) fl[nf++] = is;
      if (ir == n - 1) fl[nf++] = n + is;
      if (is == 0) fl[nf++] = 2 * n + ir;
      if (is == n - 1) fl[nf++] = 3 * n + ir;
      double rJ = base[C::O_GEO + 11];
      double rw = op.rwq[m];
      double* R = base + C::O_RXYH + 8 * m;
      int cnt = op.hg_count[m];
      // on axis-aligned elements r-line pairs and x faces feed the x half only, s-line
      // pairs and y faces the y half (gathers in the merged lists' order)
      const int fx = ir == 0 ? is : (ir == n - 1 ? n + is : -1);
      const int fy = is == 0 ? 2 * n + ir : (is == n - 1 ? 3 * n + ir : -1);
      if (aa && !(flags & F_KPP)) {
        node_half_aa<N1D, TH>(op, base, m, 0, acc64);
        node_half_aa<N1D, TH>(op, base, m, 1, acc64);
        continue;
      }
      if (sizeof(TH) == 8 || acc64) {
        double Q[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        double Bs[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        if (aa) {  // KPP: the pair terms of both axes are written (fS_kpp)
#pragma unroll
          for (int ax = 0; ax < 2; ++ax)
            for (int t = 0; t < n - 1; ++t) {
              const double* sf = base + C::O_SCR + 8 * op.hga_pair[ax][m][t];
              const int sg = op.hga_sign[ax][m][t];
#pragma unroll
              for (int c = 0; c < 4; ++c) Q[4 * ax + c] = Q[4 * ax + c] + signed_by(sf[4 * ax + c], sg);
            }
          const double* BHx = base + C::O_BFH + 8 * (fx < 0 ? 0 : fx);
          const double* BHy = base + C::O_BFH + 8 * (fy < 0 ? 0 : fy);
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            Bs[c] = fx < 0 ? 0.0 : rw * BHx[c];
            Bs[4 + c] = fy < 0 ? 0.0 : rw * BHy[4 + c];
          }
        } else {
          for (int t = 0; t < cnt; ++t) {
            const double* sf = base + C::O_SCR + 8 * op.hg_pair[m][t];
            const int sg = op.hg_sign[m][t];
#pragma unroll
            for (int c = 0; c < 8; ++c) Q[c] = Q[c] + signed_by(sf[c], sg);
          }
          for (int t = 0; t < nf; ++t) {
            const double* BH = base + C::O_BFH + 8 * fl[t];
#pragma unroll
            for (int c = 0; c < 8; ++c) Bs[c] = Bs[c] + rw * BH[c];
          }
        }
#pragma unroll
        for (int c = 0; c < 8; ++c) R[c] = (-(rw * Q[c] + Bs[c])) * rJ;
      } else {
        const float* sfb = reinterpret_cast<const float*>(base + C::O_SCR);
        const float rwf = op.rwqf[m];
        float Q[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        float Bs[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        if (aa) {
#pragma unroll
          for (int ax = 0; ax < 2; ++ax)
            for (int t = 0; t < n - 1; ++t) {
              const float* sf = sfb + 8 * op.hga_pair[ax][m][t];
              const int sg = op.hga_sign[ax][m][t];
#pragma unroll
              for (int c = 0; c < 4; ++c) Q[4 * ax + c] = Q[4 * ax + c] + signed_by(sf[4 * ax + c], sg);
            }
          const double* BHx = base + C::O_BFH + 8 * (fx < 0 ? 0 : fx);
          const double* BHy = base + C::O_BFH + 8 * (fy < 0 ? 0 : fy);
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            Bs[c] = fx < 0 ? 0.0f : rwf * (float)BHx[c];
            Bs[4 + c] = fy < 0 ? 0.0f : rwf * (float)BHy[4 + c];
          }
        } else {
          for (int t = 0; t < cnt; ++t) {
            const float* sf = sfb + 8 * op.hg_pair[m][t];
            const int sg = op.hg_sign[m][t];
#pragma unroll
            for (int c = 0; c < 8; ++c) Q[c] = Q[c] + signed_by(sf[c], sg);
          }
          for (int t = 0; t < nf; ++t) {
            const double* BH = base + C::O_BFH + 8 * fl[t];
#pragma unroll
            for (int c = 0; c < 8; ++c) Bs[c] = Bs[c] + rwf * (float)BH[c];
          }
        }
        const float rJf = reinterpret_cast<const float*>(base + C::O_GEO + 12)[4];
#pragma unroll
        for (int c = 0; c < 8; ++c) R[c] = (double)((-(rwf * Q[c] + Bs[c])) * rJf);
      }
    }
    }
  }
  __syncthreads();

  // ---- debug / non-limited outputs
  const bool dbg = flags & F_WRITE_DEBUG;
  const bool need_rhsL = dbg || (flags & F_RHSU_FROM_L);
  const bool need_rhsH = dbg || (flags & F_RHSU_FROM_H);
  if (need_rhsL && do_low) {
    for (int w = tid; w < Ke * Nq * 4; w += bs) {
      int e = w / (Nq * 4), r = w % (Nq * 4);
      a.rhsL[(size_t)k0 * Nq * 4 + w] = sm[e * PE + C::O_RHSL + r];
    }
  }
  if (need_rhsH && do_high) {
    for (int w = tid; w < Ke * Nq * 4; w += bs) {
      int e = w / (Nq * 4), r = w % (Nq * 4);
      int m = r / 4, c = r % 4;
      const double* R = sm + e * PE + C::O_RXYH + 8 * m;
      a.rhsH[(size_t)k0 * Nq * 4 + w] = R[c] + R[4 + c];
    }
  }
  if (dbg || (GAUSS && (flags & F_CELL_ENTROPY))) {
    for (int w = tid; w < Ke * Nq * 8 && dbg; w += bs) {
      int e = w / (Nq * 8), r = w % (Nq * 8);
      if (do_low) a.rhsxyL[(size_t)k0 * Nq * 8 + w] = sm[e * PE + C::O_RXYL + r];
      if (do_high) a.rhsxyH[(size_t)k0 * Nq * 8 + w] = sm[e * PE + C::O_RXYH + r];
    }
    for (int w = tid; w < Ke * Nfp * 8; w += bs) {
      int e = w / (Nfp * 8), r = w % (Nfp * 8);
      a.BFL[(size_t)k0 * Nfp * 8 + w] = sm[e * PE + C::O_BFL + r];
      a.BFH[(size_t)k0 * Nfp * 8 + w] = sm[e * PE + C::O_BFH + r];
    }
  }
  if (flags & F_ZHANG_SHU) {
    // ---- ZhangShuLimiter (zhangshu.jl:4-45): per node, the largest l in [0, 1] with
    //      uL + l P inside (zeta rhoL, zeta rhoeL, Inf, Inf), uL = U + dt rhsL,
    //      P = dt (rhsH - rhsL); L[k] = the element's min; rhsU = (1 - l) rhsL + l rhsH
    //      with l = min(L[k], blending factor)
    for (int w = tid; w < Ke * Nq; w += bs) {
      int e = w / Nq, m = w % Nq;
      double* base = sm + e * PE;
      const double* U = base + C::O_U + 4 * m;
      const double* rl = base + C::O_RHSL + 4 * m;
      const double* R = base + C::O_RXYH + 8 * m;
      double uL[4], P[4];
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        uL[c] = low_update(U[c], dt_lim, rl[c]);
        P[c] = dt_lim * ((R[c] + R[4 + c]) - rl[c]);
      }
      if (flags & F_KPP) {  // zhang_shu_bound_limiter!(::KPP) (zhangshu.jl:58-60)
        base[C::O_SCR + m] = 1.0;
        continue;
      }
      const double Lrhoe = a.zeta * fma(-0.5, (uL[1] * uL[1] + uL[2] * uL[2]) * rcp(uL[0]), uL[3]);
      double l = density_bound(uL[0], P[0], a.zeta * uL[0], __longlong_as_double(0x7ff0000000000000LL), false, 0.0);
      l = fmin(l, rhoe_quadratic_solve(uL, P, Lrhoe, a.ZEROTOL));
      base[C::O_SCR + m] = fmin(1.0, l);
    }
    __syncthreads();
    for (int e = tid; e < Ke; e += bs) {
      double* base = sm + e * PE;
      double l = 1.0;
      for (int m = 0; m < Nq; ++m) l = fmin(l, base[C::O_SCR + m]);
      a.Lelem[(size_t)(a.nstage - 1) * a.K + k0 + e] = l;
      base[C::O_SCR + Nq] = (flags & F_SHOCK) ? fmin(l, base[C::O_GEO + 15]) : l;
    }
    __syncthreads();
    for (int w = tid; w < Ke * Nq * 4; w += bs) {
      int e = w / (Nq * 4), r = w % (Nq * 4);
      int m = r / 4, c = r % 4;
      const double* base = sm + e * PE;
      const double l = base[C::O_SCR + Nq];
      const double* R = base + C::O_RXYH + 8 * m;
      a.rhsU[(size_t)k0 * Nq * 4 + w] = (1.0 - l) * base[C::O_RHSL + r] + l * (R[c] + R[4 + c]);
    }
    return;
  }
  if (!(flags & F_DO_LIMIT)) return;

  // ---- P8: subcell flux prefix sums (accumulate_f_bar!(::Dim2), subcell.jl:163-206)
  //          and the low-order update uL = U + dt*rhsL (subcell.jl:269)
  // Item (e, d, line l, c); x lines (d = 0, line sj) start at face sj and run through
  // faces si + (n+1) sj and nodes (si-1) + n sj; y lines (d = 1, line si) start at face
  // 2n + si and run through faces si + n sj and nodes si + n (sj-1). Both as strides, so
  // a warp's x and y items share every instruction.
  for (int w = tid; w < Ke * 8 * n; w += bs) {
    int e = w / (8 * n), r = w % (8 * n);
    int d = r / (4 * n), l = (r / 4) % n, c = r % 4;
    double* base = sm + e * PE;
    const double* wJq = base + C::O_WS;  // wq J per node, 2 apart
    double* fb = base + C::O_SCR;  // [d][HL][face][c]
    double* fH = fb + (d * 2 + 0) * NSF * 4;
    double* fL = fb + (d * 2 + 1) * NSF * 4;
    const int f0 = d == 0 ? l : 2 * n + l;       // boundary face where the line starts
    const int fs = d == 0 ? 1 : n, fb0 = d == 0 ? (n + 1) * l : l;  // subcell faces
    const int qs = d == 0 ? 1 : n, qb0 = d == 0 ? n * l : l;        // nodes
    const int o = 4 * d + c;
    double h = base[C::O_BFH + 8 * f0 + o], lo = base[C::O_BFL + 8 * f0 + o];
    fH[fb0 * 4 + c] = h;
    fL[fb0 * 4 + c] = lo;
    for (int t = 1; t <= n; ++t) {
      const int q = qb0 + qs * (t - 1);
      const double wJ = wJq[2 * q];
      h = h + wJ * base[C::O_RXYH + 8 * q + o];
      lo = lo + wJ * base[C::O_RXYL + 8 * q + o];
      fH[(fb0 + fs * t) * 4 + c] = h;
      fL[(fb0 + fs * t) * 4 + c] = lo;
    }
  }
  for (int w = tid; w < Ke * Nq; w += bs) {
    int e = w / Nq, m = w % Nq;
    double* base = sm + e * PE;
    const double* U = base + C::O_U + 4 * m;
    const double* rl = base + C::O_RHSL + 4 * m;
    double* uL = base + C::O_PRIM + 6 * m;
#pragma unroll
    for (int c = 0; c < 4; ++c) uL[c] = low_update(U[c], dt_lim, rl[c]);
    uL[4] = a.zeta * fma(-0.5, (uL[1] * uL[1] + uL[2] * uL[2]) * rcp(uL[0]), uL[3]);  // zeta rhoe_ufun(uL)
    uL[5] = (4.0 * dt_lim) * base[C::O_WS + 2 * m + 1];  // 4 dt / (wq J)
    // density bounds (rho_bound, subcell.jl:352-387): Lrho, rho/2, Urho (rl is read above)
    double* lim = base + C::O_RHSL + 4 * m;
    const int ir = m % n, is = m / n, k = k0 + e;
    // global node index of stencil member t of low_order_stencil (limiter_utils.jl:222-231):
    // r-neighbours, then s-neighbours, across a face through quad_index_to_quad_index_P
    // (:199-212), whose q2fq lists the r-face first
    auto stencil = [&](int t) -> size_t {
      const int dir = t >> 1, up = t & 1;  // 0: r, 1: s; lower or upper neighbour
      const int c = dir == 0 ? ir : is;
      if (up ? c < n - 1 : c > 0) return (size_t)k * Nq + m + (dir == 0 ? 1 : n) * (up ? 1 : -1);
      // the face of this node in direction dir (a node on one face has only that one)
      int f;
      if (dir == 0 && (ir == 0 || ir == n - 1)) f = ir == 0 ? is : n + is;
      else if (dir == 1 && (is == 0 || is == n - 1)) f = is == 0 ? 2 * n + ir : 3 * n + ir;
      else f = ir == 0 ? is : (ir == n - 1 ? n + is : (is == 0 ? 2 * n + ir : 3 * n + ir));
      const int lin = a.nbr[(size_t)k * Nfp + f];
      const int kP = lin / Nfp, iP = lin % Nfp, sP = iP / n, tP = iP % n;
      const int qP = sP == 0 ? n * tP : sP == 1 ? (n - 1) + n * tP : sP == 2 ? tP : tP + n * (n - 1);
      return (size_t)kP * Nq + qP;
    };
    if (flags & F_TVD) {
      // min/max of the low-order density over the node and its stencil (subcell.jl:112-141)
      const double* rl_g = a.rhoL;
      double lb = rl_g[(size_t)k * Nq + m], ub = lb;
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        const double v = rl_g[stencil(t)];
        lb = fmin(lb, v);
        ub = fmax(ub, v);
      }
      lim[0] = lb;
      lim[2] = ub;
    } else {
      lim[0] = a.zeta * uL[0];
      lim[2] = __longlong_as_double(0x7ff0000000000000LL);
    }
    if (flags & F_MIN_ENTROPY) {
      // initialize_lower_bound!(::Dim2) (subcell.jl:53-72): Lphi = eps_k min(phi over the
      // node and its stencil) + (1 - eps_k) phi_min; eps_k = 1 unless relaxed; the
      // bisection's threshold Lphi - POSTOL in lim[3]
      double lb = s_modified(U[0], U[1], U[2], U[3], a.gamma);
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        const double* Un = a.Uq + 4 * stencil(t);
        lb = fmin(lb, s_modified(Un[0], Un[1], Un[2], Un[3], a.gamma));
      }
      if (flags & F_RELAXED) {
        const double eps = base[C::O_XT];
        lb = eps * lb + (1 - eps) * a.phimin[0];
      }
      lim[3] = lb - a.POSTOL;
    }
    lim[1] = 0.5 * uL[0];
  }
  __syncthreads();

  // ---- P9: bound evaluations, four per node (subcell_bound_limiter!(::Dim2), :288-341).
  // Evaluation r = (2d + h) Nq + m limits face h (0: lower, 1: upper) of node m in
  // direction d with P = -/+ 4 dt (fH - fL) / (wq J). A face's factor is the min of its
  // one or two evaluations. First the density bound of every evaluation (it needs only
  // P[0]); the quadratic internal-energy solve (>= ZEROTOL or 1, never NaN) can only
  // change the face's factor when every density bound of that face is nonzero, so only
  // those evaluations go to a list, solved with all lanes busy.
  // the 5-tuple bound (Lrho, Lrhoe, Lphi = 0, Urho_i, Urhoe = Inf) read as 4 names under
  // the reference semantics: Urho = 0 and Urhoe = Urho_i (limiter_utils.jl:66-70).
  // KPP evaluates no bound (subcell_bound_limiter!(dim, ::KPP), subcell.jl:389-402).
  if (!(flags & F_KPP)) {
  const bool upper0 = flags & F_REF_SEM;
  for (int w = tid; w < Ke * NEV; w += bs) {
    int e = w / NEV, r = w % NEV;
    int dh = r / Nq, m = r % Nq;
    int ir = m % n, is = m / n;
    double* base = sm + e * PE;
    const double* fb = base + C::O_SCR;
    int d = dh >> 1, h = dh & 1;
    int fi = (d == 0) ? (ir + h) + (n + 1) * is : ir + n * (is + h);
    const double* fH = fb + ((d * 2 + 0) * NSF + fi) * 4;
    const double* fL = fb + ((d * 2 + 1) * NSF + fi) * 4;
    const double* uL = base + C::O_PRIM + 6 * m;
    double P0 = (fH[0] - fL[0]) * uL[5];
    if (h == 0) P0 = -P0;
    const double* lim = base + C::O_RHSL + 4 * m;
    base[C::O_EV + r] = density_bound(uL[0], P0, lim[0], upper0 ? 0.0 : lim[2], upper0, lim[1]);
  }
  __syncthreads();
  for (int w = tid; w < Ke * NEV; w += bs) {
    int e = w / NEV, r = w % NEV;
    int dh = r / Nq, m = r % Nq;
    int ir = m % n, is = m / n;
    const double* ev = sm + e * PE + C::O_EV;
    if (is_zero_bits(ev[r])) continue;
    int d = dh >> 1, h = dh & 1;
    // the other evaluation of the same face, if the face is interior
    int partner = -1;
    if (d == 0) {
      if (h == 0 && ir > 0) partner = 1 * Nq + (ir - 1) + n * is;
      if (h == 1 && ir + 1 < n) partner = 0 * Nq + (ir + 1) + n * is;
    } else {
      if (h == 0 && is > 0) partner = 3 * Nq + ir + n * (is - 1);
      if (h == 1 && is + 1 < n) partner = 2 * Nq + ir + n * (is + 1);
    }
    if (partner >= 0 && is_zero_bits(ev[partner])) continue;
    int slot = atomicAdd(&s_list[0], 1);
    s_list[1 + slot] = e * NEV + r;
  }
  __syncthreads();
  const int nlist = s_list[0];
  for (int w = tid; w < nlist; w += bs) {
    int id = s_list[1 + w];
    int e = id / NEV, r = id % NEV;
    int dh = r / Nq, m = r % Nq;
    int ir = m % n, is = m / n;
    int d = dh >> 1, h = dh & 1;
    double* base = sm + e * PE;
    const double* fb = base + C::O_SCR;
    int fi = (d == 0) ? (ir + h) + (n + 1) * is : ir + n * (is + h);
    const double* fH = fb + ((d * 2 + 0) * NSF + fi) * 4;
    const double* fL = fb + ((d * 2 + 1) * NSF + fi) * 4;
    const double* uL = base + C::O_PRIM + 6 * m;
    double P[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      double t = (fH[c] - fL[c]) * uL[5];
      P[c] = h == 0 ? -t : t;
    }
    double l = base[C::O_EV + r];
    l = fmin(l, rhoe_quadratic_solve(uL, P, uL[4], a.ZEROTOL));
    // the second solve of limiting_param_bound_rho_rhoe: Urhoe = Urho_i (the TVD upper
    // density bound) under the reference semantics, else Inf, for which it returns 1.0
    const double Urhoe = upper0 ? base[C::O_RHSL + 4 * m + 2] : __longlong_as_double(0x7ff0000000000000LL);
    if (upper0 && (flags & F_TVD)) l = fmin(l, rhoe_quadratic_solve(uL, P, Urhoe, a.ZEROTOL));
    // min-entropy bounds (limiter_utils.jl:19-24): l is lpos, then the bisection. Its first
    // test (at lpos) runs here; an evaluation that fails it goes, with lpos, to a second list
    // whose 21 halvings run below with every lane busy (a warp issues each pow of the loop
    // once for all its lanes, so a few bisecting lanes among finished ones would cost the
    // warp the whole loop). The list lives in the low-order rhsxy region, dead after P8.
    if (flags & F_MIN_ENTROPY) {
      if (!phi_at_least(uL, P, l, base[C::O_RHSL + 4 * m + 3], a.gamma)) {
        base[C::O_EV + r] = l;
        const int slot = atomicAdd(&s_list[NEV * E + 1], 1);
        bisect_slot<C>(sm, PE, slot) = id;
        continue;
      }
    }
    base[C::O_EV + r] = fmin(l, 1.0);
  }
  if (a.counters && tid == 0 && nlist) atomicAdd(&a.counters[0], (unsigned long long)nlist);
  __syncthreads();
  if (flags & F_MIN_ENTROPY) {
    const int nbis = s_list[NEV * E + 1];
    for (int w = tid; w < nbis; w += bs) {
      const int id = bisect_slot<C>(sm, PE, w);
      const int e = id / NEV, r = id % NEV;
      const int dh = r / Nq, m = r % Nq;
      const int ir = m % n, is = m / n;
      const int d = dh >> 1, h = dh & 1;
      double* base = sm + e * PE;
      const double* fb = base + C::O_SCR;
      const int fi = (d == 0) ? (ir + h) + (n + 1) * is : ir + n * (is + h);
      const double* fH = fb + ((d * 2 + 0) * NSF + fi) * 4;
      const double* fL = fb + ((d * 2 + 1) * NSF + fi) * 4;
      const double* uL = base + C::O_PRIM + 6 * m;
      double P[4];
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        double t = (fH[c] - fL[c]) * uL[5];
        P[c] = h == 0 ? -t : t;
      }
      const double l = bisect_phi_halvings(uL, P, base[C::O_EV + r], base[C::O_RHSL + 4 * m + 3], a.gamma);
      base[C::O_EV + r] = fmin(l, 1.0);
    }
    __syncthreads();
  }
  }

  // ---- P10: combine evaluations per subcell face; blending factor 1 (NoShockCapture)
  for (int w = tid; w < Ke * 2 * NSF; w += bs) {
    int e = w / (2 * NSF), r = w % (2 * NSF);
    int d = r / NSF, fi = r % NSF;
    double* base = sm + e * PE;
    const double* ev = base + C::O_EV;
    // 1, or the element's shock-capture blending factor (the final min of subcell.jl:345)
    double L = (flags & F_SHOCK) ? base[C::O_GEO + 15] : 1.0;
    if (flags & F_KPP) {  // min(1, blending factor)
      base[C::O_L + r] = fmin(1.0, L);
      continue;
    }
    if (d == 0) {
      int si = fi % (n + 1), sj = fi / (n + 1);
      if (si < n) L = min_nonneg_bits(L, ev[0 * Nq + si + n * sj]);
      if (si > 0) L = min_nonneg_bits(L, ev[1 * Nq + (si - 1) + n * sj]);
    } else {
      int si = fi % n, sj = fi / n;
      if (sj < n) L = min_nonneg_bits(L, ev[2 * Nq + si + n * sj]);
      if (sj > 0) L = min_nonneg_bits(L, ev[3 * Nq + si + n * (sj - 1)]);
    }
    base[C::O_L + r] = L;
  }
  __syncthreads();

  // ---- P11: cell entropy bound (enforce_ES_subcell!, subcell.jl:462-744)
  // Every product and sum of this phase is an explicitly rounded operation (__dmul_rn,
  // __dadd_rn, ...), none left for the compiler to contract into an FMA: the greedy below
  // amplifies a one-ulp change of its inputs, and a contraction chosen differently in the
  // batch kernel than in the single-solve kernel would give a batch member other bits
  // than its solo run. The sums follow the oracle's order, unfused as there. The per-face
  // products run one item per face (P11c) on all lanes; only the ordered sums, the sort
  // and the greedy run per element and direction (P11d).
  if (flags & F_CELL_ENTROPY) {
    constexpr int M = Nq - n;  // interior subcell faces per direction
    // scratch in the primitives region (uL is dead after P9): dvdf [2][M], sum_c dv fL
    // [2][M], B psi [2][Nfp]
    constexpr int O_DV = C::O_PRIM, O_DL = O_DV + 2 * M, O_BP = O_DL + 2 * M;
    static_assert(4 * M + 2 * Nfp <= 6 * Nq, "cell-entropy scratch fits the primitives region");
    // and in the low-order rhsxy region (dead after P8): the sort keys of dvdf [2][M]
    // (long long) and the sorted order [2][M] (int)
    constexpr int O_KEY = C::O_RXYL, O_ORD = O_KEY + 2 * M;
    static_assert(3 * M <= 8 * Nq, "sort scratch fits the low-order rhsxy region");
    // An element-direction whose interior factors are all zero has sum(L*dvdf) = 0
    // (or NaN) and the check of subcell.jl:676-677 is false: nothing to do.
    for (int w = tid; w < Ke * 2; w += bs) {
      int e = w / 2, d = w % 2;
      double* base = sm + e * PE;
      const double* L = base + C::O_L + d * NSF;
      bool any = false;
      for (int sj = 0; sj < n; ++sj)
        for (int si = 1; si < n; ++si) {
          double v = d == 0 ? L[si + (n + 1) * sj] : L[sj + n * si];
          if (!is_zero_bits(v)) any = true;
        }
      base[C::O_MISC + d] = any ? 1.0 : 0.0;
    }
    __syncthreads();
    // P11b: entropy variables v_ufun (compressible_Navier_Stokes.jl:134-144) at the nodes
    // of the elements that need them; s = log(p) - gamma log(rho) for log(p / rho^gamma)
    for (int w = tid; w < Ke * Nq; w += bs) {
      int e = w / Nq, m = w % Nq;
      double* base = sm + e * PE;
      if (is_zero_bits(base[C::O_MISC]) && is_zero_bits(base[C::O_MISC + 1])) continue;
      const double* U = base + C::O_U + 4 * m;
      const double ke = __dadd_rn(__dmul_rn(U[1], U[1]), __dmul_rn(U[2], U[2]));
      const double p = __dmul_rn(a.gm1, __dsub_rn(U[3], __ddiv_rn(__dmul_rn(0.5, ke), U[0])));
      const double s = __dsub_rn(log_fast(p, op), __dmul_rn(a.gamma, log_fast(U[0], op)));
      const double rp = rcp(p);
      double* vq = base + C::O_FLUX + 4 * m;
      vq[0] = __dsub_rn(__dsub_rn(__dadd_rn(a.gamma, 1.0), s), __dmul_rn(__dmul_rn(a.gm1, U[3]), rp));
      vq[1] = __dmul_rn(__dmul_rn(U[1], a.gm1), rp);
      vq[2] = __dmul_rn(__dmul_rn(U[2], a.gm1), rp);
      vq[3] = __dmul_rn(__dmul_rn(-U[0], a.gm1), rp);
    }
    __syncthreads();
    // P11c: per interior face, dvdf = sum_c dv_c (fH - fL)_c, its sort key (Julia's
    // isless order as an integer: NaN above everything, -0 below +0) and sum_c dv_c fL_c
    // (subcell.jl:540-562); per face node, B psi (:521-529). dvdf index of a face: x,
    // (si-1) + (n-1) sj; y, si + n (sj-1).
    for (int w = tid; w < Ke * 2 * (M + Nfp); w += bs) {
      const int e = w / (2 * (M + Nfp)), r = w % (2 * (M + Nfp));
      const int d = r / (M + Nfp), j = r % (M + Nfp);
      double* base = sm + e * PE;
      if (is_zero_bits(base[C::O_MISC + d])) continue;
      if (j < M) {
        int fi, qm, qp;
        if (d == 0) {
          const int si = j % (n - 1) + 1, sj = j / (n - 1);
          fi = si + (n + 1) * sj;
          qm = (si - 1) + n * sj;
          qp = si + n * sj;
        } else {
          const int si = j % n, sj = j / n + 1;
          fi = si + n * sj;
          qm = si + n * (sj - 1);
          qp = si + n * sj;
        }
        const double* vq = base + C::O_FLUX;
        const double* fH = base + C::O_SCR + (d * 2 + 0) * NSF * 4 + fi * 4;
        const double* fL = base + C::O_SCR + (d * 2 + 1) * NSF * 4 + fi * 4;
        double pr_d[4], pr_l[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          const double dv = __dsub_rn(vq[4 * qm + c], vq[4 * qp + c]);
          pr_d[c] = __dmul_rn(dv, __dsub_rn(fH[c], fL[c]));
          pr_l[c] = __dmul_rn(dv, fL[c]);
        }
        const double dvdf = __dadd_rn(__dadd_rn(__dadd_rn(pr_d[0], pr_d[1]), pr_d[2]), pr_d[3]);
        base[O_DV + d * M + j] = dvdf;
        base[O_DL + d * M + j] = __dadd_rn(__dadd_rn(__dadd_rn(pr_l[0], pr_l[1]), pr_l[2]), pr_l[3]);
        const long long bits = __double_as_longlong(dvdf);
        reinterpret_cast<long long*>(base + O_KEY)[d * M + j] =
            (bits & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL ? 0x7fffffffffffffffLL : order_key(dvdf);
      } else {
        const int f = j - M, side = f / n, tt = f % n;
        const int q = side == 0 ? n * tt : side == 1 ? (n - 1) + n * tt : side == 2 ? tt : tt + n * (n - 1);
        const double* G = base + C::O_GEO;
        const double Br = side == 0 ? -op.w1D[tt] : side == 1 ? op.w1D[tt] : 0.0;
        const double Bsv = side == 2 ? -op.w1D[tt] : side == 3 ? op.w1D[tt] : 0.0;
        const double Bd = d == 0 ? __dadd_rn(__dmul_rn(G[1], Br), __dmul_rn(G[2], Bsv))
                                 : __dadd_rn(__dmul_rn(G[3], Br), __dmul_rn(G[4], Bsv));
        base[O_BP + d * Nfp + f] = __dmul_rn(Bd, __dmul_rn(a.gm1, base[C::O_U + 4 * q + 1 + d]));
      }
    }
    __syncthreads();
    // P11e: the descending sort of (dvdf, index) as ranks, one item per face: the faces
    // that sort before face i are those with a larger key, or an equal key and a larger
    // index (sort!(rev = true) on the (value, index) tuples, subcell.jl:676-741)
    for (int w = tid; w < Ke * 2 * M; w += bs) {
      const int e = w / (2 * M), r = w % (2 * M), d = r / M, i = r % M;
      double* base = sm + e * PE;
      if (is_zero_bits(base[C::O_MISC + d])) continue;
      const long long* key = reinterpret_cast<const long long*>(base + O_KEY) + d * M;
      const long long ki = key[i];
      int rank = 0;
#pragma unroll
      for (int j = 0; j < M; ++j) rank += (key[j] > ki || (key[j] == ki && j > i)) ? 1 : 0;
      reinterpret_cast<int*>(base + O_ORD)[d * M + rank] = i;
    }
    __syncthreads();
    // P11d: per element and direction, the sums in the oracle's order, rhs_es and the greedy
    for (int w = tid; w < Ke * 2; w += bs) {
      int e = w / 2, d = w % 2;
      double* base = sm + e * PE;
      if (is_zero_bits(base[C::O_MISC + d])) continue;
      double* L = base + C::O_L + d * NSF;
      // sum_Bpsi over all face nodes in order
      double sB = 0.0;
      for (int f = 0; f < Nfp; ++f) sB = __dadd_rn(sB, base[O_BP + d * Nfp + f]);
      const double* dvdf = base + O_DV + d * M;
      // sum_dvfbarL and sum of L*dvdf (subcell.jl:540-562, 654-670) in the reference loop
      // order: x: line sj outer, face si = 1..n-1 inner; y: line si outer, face sj inner
      double sdl = 0.0, sumLd = 0.0;
      for (int a2 = 0; a2 < n; ++a2)
        for (int b2 = 1; b2 < n; ++b2) {
          const int fi = d == 0 ? b2 + (n + 1) * a2 : a2 + n * b2;
          const int idx = d == 0 ? (b2 - 1) + (n - 1) * a2 : a2 + n * (b2 - 1);
          sdl = __dadd_rn(sdl, base[O_DL + d * M + idx]);
          sumLd = __dadd_rn(sumLd, __dmul_rn(L[fi], dvdf[idx]));
        }
      double rhs = __dsub_rn(sB, sdl);
      // rhs_es of the relaxed bounds (subcell.jl:750-753)
      if (flags & F_RELAXED) rhs = __dmul_rn(__dsub_rn(1.0, __dmul_rn(a.beta, base[C::O_XT])), rhs);
      double est = __dsub_rn(sumLd, rhs);
      double tol = jmax(0.0, __dsub_rn(sdl, sB));
      if (est > tol) {
        const int* ord = reinterpret_cast<const int*>(base + O_ORD) + d * M;
        auto face_of_idx = [&](int idx) {  // 0-based dvdf index -> L face index
          if (d == 0) {
            int si = idx % (n - 1) + 1, sj = idx / (n - 1);
            return si + (n + 1) * sj;
          }
          int si = idx % n, sj = idx / n + 1;
          return si + n * sj;
        };
        int curr = 0;
        double lhs = sumLd;
        const double target = __dadd_rn(rhs, tol);
        while (lhs > target && curr < M) {
          int idx = ord[curr];
          if (dvdf[idx] < a.ZEROTOL) break;
          lhs = __dsub_rn(lhs, __dmul_rn(L[face_of_idx(idx)], dvdf[idx]));
          ++curr;
        }
        for (int i2 = 0; i2 < curr; ++i2) {
          int idx = ord[i2];
          int fi = face_of_idx(idx);
          double l_new = (i2 == curr - 1) ? jmax(__ddiv_rn(__dsub_rn(target, lhs), dvdf[idx]), 0.0) : 0.0;
          L[fi] = jmin(L[fi], l_new);
        }
      }
    }
    __syncthreads();
  }

  // ---- P12: L before symmetrization and the subcell fluxes for kernel B
  for (int w = tid; w < Ke * 2 * NSF; w += bs) {
    int e = w / (2 * NSF), r = w % (2 * NSF);
    a.Lpre[(size_t)(k0 + e) * 2 * NSF + r] = sm[e * PE + C::O_L + r];
  }
  for (int w = tid; w < Ke * C::FBAR; w += bs) {
    int e = w / C::FBAR, r = w % C::FBAR;
    a.fbar[(size_t)(k0 + e) * C::FBAR + r] = sm[e * PE + C::O_SCR + r];
  }
}

template <int N1D, typename TH, bool GAUSS = false, bool EXT = false>
__global__ void __launch_bounds__(Cfg<N1D>::THREADS) k_stage_a(StageArgs a) {
  extern __shared__ __align__(16) double sm[];
  stage_a_body<N1D, TH, GAUSS, EXT>(a, blockIdx.x * a.epb, sm);
}

// =====================================================================================
// Kernel B: symmetrize, blend, rhsU, SSP-RK3 stage update
// =====================================================================================
// Body of kernel B for the elements k0 .. k0+E-1 of the solve `a`; the block holding
// element 0 also advances the solve's dt and t.
template <int N1D>
__device__ __forceinline__ void stage_b_body(const StageArgs& a, int k0, double* sm) {
  using C = Cfg<N1D>;
  constexpr int n = C::n, Nq = C::Nq, Nfp = C::Nfp, NSF = C::NSF;
  constexpr int PE = C::PER_ELEM_B;
  if (a.scal[S_DONE] != 0.0) return;
  const OpTable& op = *a.ops;
  const int tid = threadIdx.x, bs = blockDim.x;
  const int Ke = min(a.epb, a.K - k0);
  if (Ke <= 0) return;
  const int flags = a.flags;
  const int s = a.nstage - 1;
  double dt;
  if (a.nstage == 1 && (flags & F_UPDATE))
    dt = __longlong_as_double((long long)*a.dtmin_bits);
  else
    dt = a.scal[S_DT];
  const bool limited = flags & F_DO_LIMIT;
  // smem: L [2 NSF], fbar [16 NSF], flim [8 NSF], 1/J
  if (limited) {
    for (int e = tid; e < Ke; e += bs) sm[e * PE + 26 * NSF] = rcp(a.geom[5 * (size_t)(k0 + e)]);
    for (int w = tid; w < Ke * 2 * NSF; w += bs) {
      int e = w / (2 * NSF), r = w % (2 * NSF);
      sm[e * PE + r] = a.Lpre[(size_t)(k0 + e) * 2 * NSF + r];
    }
    for (int w = tid; w < Ke * C::FBAR; w += bs) {
      int e = w / C::FBAR, r = w % C::FBAR;
      sm[e * PE + 2 * NSF + r] = a.fbar[(size_t)(k0 + e) * C::FBAR + r];
    }
    __syncthreads();
    // symmetrize_limiting_parameters!(::Dim2) with subcell_index_P_x/y (limiter_utils.jl:179-237)
    for (int w = tid; w < Ke * 4 * n; w += bs) {
      int e = w / (4 * n), r = w % (4 * n);
      int d = r / (2 * n), side = (r / n) % 2, tt = r % n;
      const int k = k0 + e;
      int iface, idx;
      if (d == 0) {
        iface = side ? tt + n : tt;
        idx = (side ? n : 0) + (n + 1) * tt;
      } else {
        iface = side ? tt + 3 * n : tt + 2 * n;
        idx = tt + n * (side ? n : 0);
      }
      int lin = a.nbr[(size_t)k * Nfp + iface];
      int kP = lin / Nfp, iP = lin % Nfp;
      int idxP;
      if (d == 0) {
        int sjP = iP % n;
        int siP = (iP / n == 0) ? 0 : n;
        idxP = siP + (n + 1) * sjP;
      } else {
        int siP = iP % n;
        int sjP = (iP / n == 2) ? 0 : n;
        idxP = siP + n * sjP;
      }
      double own = a.Lpre[(size_t)k * 2 * NSF + d * NSF + idx];
      double par = a.Lpre[(size_t)kP * 2 * NSF + d * NSF + idxP];
      sm[e * PE + d * NSF + idx] = fmin(own, par);
    }
    __syncthreads();
    // accumulate_f_bar_limited!(::Dim2) (subcell.jl:841-876)
    for (int w = tid; w < Ke * 2 * NSF * 4; w += bs) {
      int e = w / (2 * NSF * 4), r = w % (2 * NSF * 4);
      int d = r / (NSF * 4), fi = (r / 4) % NSF, c = r % 4;
      double* base = sm + e * PE;
      double l = base[d * NSF + fi];
      const double* fb = base + 2 * NSF;
      double fH = fb[((d * 2 + 0) * NSF + fi) * 4 + c];
      double fL = fb[((d * 2 + 1) * NSF + fi) * 4 + c];
      // l fH + (1 - l) fL as fL + l (fH - fL): one rounding fewer, and exactly fL at l = 0
      base[2 * NSF + 16 * NSF + (d * NSF + fi) * 4 + c] = fma(l, fH - fL, fL);
    }
    __syncthreads();
  }
  // apply_subcell_limiter!(::Dim2) (subcell.jl:894-924) and the stage combination
  // minima as ordered integer keys (integer pipe)
  long long rmin = order_key(__longlong_as_double(0x7ff0000000000000LL)), emin = rmin;
  for (int w = tid; w < Ke * Nq; w += bs) {
    int e = w / Nq, m = w % Nq;
    const int k = k0 + e;
    int ir = m % n, is = m / n;
    double ru[4];
    size_t gidx = ((size_t)k * Nq + m) * 4;
    if (limited) {
      const double* fl = sm + e * PE + 2 * NSF + 16 * NSF;
      double rwJ = sm[e * PE + 26 * NSF] * op.rwq[m];  // (1/J)(1/wq)
      const double* fx0 = fl + ((0 * NSF) + ir + (n + 1) * is) * 4;
      const double* fx1 = fl + ((0 * NSF) + ir + 1 + (n + 1) * is) * 4;
      const double* fy0 = fl + ((1 * NSF) + ir + n * is) * 4;
      const double* fy1 = fl + ((1 * NSF) + ir + n * (is + 1)) * 4;
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        double x = (fx1[c] - fx0[c]) * rwJ;
        double y = (fy1[c] - fy0[c]) * rwJ;
        ru[c] = x + y;
      }
    } else if (flags & F_RHSU_FROM_L) {
#pragma unroll
      for (int c = 0; c < 4; ++c) ru[c] = a.rhsL[gidx + c];
    } else if (flags & F_ZHANG_SHU) {
#pragma unroll
      for (int c = 0; c < 4; ++c) ru[c] = a.rhsU[gidx + c];
    } else {
#pragma unroll
      for (int c = 0; c < 4; ++c) ru[c] = a.rhsH[gidx + c];
    }
#pragma unroll
    for (int c = 0; c < 4; ++c) a.rhsU[gidx + c] = ru[c];
    if (flags & F_UPDATE) {
      double U[4];
#pragma unroll
      for (int c = 0; c < 4; ++c) U[c] = a.Uq[gidx + c];
      if (a.nstage == 1) {
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          a.resW[gidx + c] = U[c];
          U[c] = U[c] + dt * ru[c];
        }
      } else if (a.nstage == 2) {
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          double z = U[c] + dt * ru[c];
          U[c] = 3.0 / 4.0 * a.resW[gidx + c] + 1.0 / 4.0 * z;
        }
      } else {
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          double z = U[c] + dt * ru[c];
          U[c] = 1.0 / 3.0 * a.resW[gidx + c] + 2.0 / 3.0 * z;
        }
      }
#pragma unroll
      for (int c = 0; c < 4; ++c) a.Uq[gidx + c] = U[c];
      double re = fma(-0.5, (U[1] * U[1] + U[2] * U[2]) * rcp(U[0]), U[3]);  // rhoe_ufun(U)
      long long kr = order_key(U[0]), ke = order_key(re);
      rmin = kr < rmin ? kr : rmin;
      emin = ke < emin ? ke : emin;
      // not (> 0): -0, negative or NaN, i.e. bits <= 0 or above +Inf's; KPP has no positivity
      if (!(flags & F_KPP) &&
          (__double_as_longlong(U[0]) <= 0 || __double_as_longlong(U[0]) > 0x7ff0000000000000LL ||
           __double_as_longlong(re) <= 0 || __double_as_longlong(re) > 0x7ff0000000000000LL))
        atomicOr(a.status, ST_NOT_POSITIVE);
    }
  }
  if (limited) {
    for (int w = tid; w < Ke * 2 * NSF; w += bs) {
      int e = w / (2 * NSF), r = w % (2 * NSF);
      a.Lfin[((size_t)s * a.K + k0 + e) * 2 * NSF + r] = sm[e * PE + r];
    }
  }
  if (flags & F_UPDATE) {
    for (int o = 16; o > 0; o >>= 1) {
      long long x = __shfl_xor_sync(0xffffffffu, rmin, o), y = __shfl_xor_sync(0xffffffffu, emin, o);
      rmin = x < rmin ? x : rmin;
      emin = y < emin ? y : emin;
    }
    if ((tid & 31) == 0) {
      atomicMin(&a.minrec[2 * s + 0], rmin);
      atomicMin(&a.minrec[2 * s + 1], emin);
    }
    if (k0 == 0 && tid == 0) {
      if (a.nstage == 1) {
        a.scal[S_DT] = dt;
        a.scal[S_DT_LIM] = dt;
      }
      if (a.nstage == 3) {
        a.scal[S_T] = a.scal[S_T] + dt;
        a.scal[S_STEPS] = a.scal[S_STEPS] + 1.0;
      }
    }
  }
}

template <int N1D>
__global__ void __launch_bounds__(Cfg<N1D>::THREADS) k_stage_b(StageArgs a) {
  extern __shared__ __align__(16) double sm[];
  stage_b_body<N1D>(a, blockIdx.x * a.epb, sm);
}

}  // namespace p2de
