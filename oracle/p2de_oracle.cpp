// p2de_oracle.cpp — TEST INFRASTRUCTURE ONLY (the parity checker and the timed CPU
// baseline). Nothing in the product links, loads or calls this file.
//
// A CPU FP64 restatement of P2DE.jl's 2D compressible-Euler DG path:
//   rhs!(::LimitedDG)            src/dg/rhs/rhs.jl:41-55
//   rhs_low_graph_visc!          src/dg/rhs/low_order_graph_viscosity.jl:4-41
//   rhs_fluxdiff!                src/dg/rhs/flux_differencing.jl:4-37
//   apply_rhs_limiter!(Subcell)  src/dg/limiter/limiter.jl:20-56, subcell.jl, limiter_utils.jl
//   apply_rhs_limiter!(ZhangShu) src/dg/limiter/limiter.jl:8-18, zhangshu.jl
//   SSP33!                       src/timestepping/SSPRK33.jl:1-62
// with the operators of initialize_operators (src/dg/init.jl:133-228) rebuilt from
// the GLL rule for tensor-product quads. Loop orders, association orders and the
// dense-operator forms of the reference are kept so that the restatement follows
// the reference operation by operation (compiled with -ffp-contract=off).
//
// PARITY UNPINNED: P2DE.jl ships no golden vectors or known-answer tests for this
// path (test/test_smoke.jl asserts nothing numeric), Julia is not available to run
// the reference, and the operator/mesh construction lives in the un-vendored
// StartUpDG (compat 0.15-0.17) and NodesAndModes (0.9) packages. The restatement is
// checked against mathematical invariants instead (SBP property, free-stream
// preservation, conservation, fS(u,u) = f(u), isentropic-vortex convergence).
//
// Parallelism mirrors Polyester's @batch over elements with OpenMP.

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <initializer_list>
#include <string>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/p2de.h"

namespace {

using V4 = std::array<double, 4>;
struct V2x4 {
  V4 x, y;
};

const double kInf = INFINITY;

// Julia's min/max on Float64: NaN propagates; -0.0 < 0.0.
inline double jmin(double x, double y) {
  if (std::isnan(x) || std::isnan(y)) return NAN;
  if (x == y) return std::signbit(x) ? x : y;
  return x < y ? x : y;
}
inline double jmax(double x, double y) {
  if (std::isnan(x) || std::isnan(y)) return NAN;
  if (x == y) return std::signbit(x) ? y : x;
  return x > y ? x : y;
}
// Julia's isless total order on Float64 (used by sort! of (value, index) tuples):
// -Inf < ... < -0.0 < 0.0 < ... < Inf < NaN.
inline bool jisless(double a, double b) {
  if (std::isnan(a)) return false;
  if (std::isnan(b)) return true;
  if (a < b) return true;
  if (a == b) return std::signbit(a) && !std::signbit(b);
  return false;
}

inline V4 add(const V4& a, const V4& b) { return {a[0] + b[0], a[1] + b[1], a[2] + b[2], a[3] + b[3]}; }
inline V4 sub(const V4& a, const V4& b) { return {a[0] - b[0], a[1] - b[1], a[2] - b[2], a[3] - b[3]}; }
inline V4 scal(double s, const V4& a) { return {s * a[0], s * a[1], s * a[2], s * a[3]}; }
inline V4 divs(const V4& a, double s) { return {a[0] / s, a[1] / s, a[2] / s, a[3] / s}; }
inline V4 neg(const V4& a) { return {-a[0], -a[1], -a[2], -a[3]}; }
// StaticArrays sum of an SVector{4}: left fold.
inline double vsum(const V4& a) { return ((a[0] + a[1]) + a[2]) + a[3]; }
inline V4 vmul(const V4& a, const V4& b) { return {a[0] * b[0], a[1] * b[1], a[2] * b[2], a[3] * b[3]}; }

// ---------------------------------------------------------------------------
// Physics: src/math/compressible_Navier_Stokes.jl (Dim2 unless noted)
// ---------------------------------------------------------------------------
struct Euler {
  double gamma;
  bool kpp = false;  // KPP{Dim2} (src/math/KPP.jl): the scalar in component 0, the rest 0

  // :24-28
  double pfun(const V4& U) const {
    return (gamma - 1.0) * (U[3] - 0.5 * (U[1] * U[1] + U[2] * U[2]) / U[0]);
  }
  // :18-22 (Dim1: rho, rhou, E)
  double pfun1(double rho, double rhou, double E) const { return (gamma - 1.0) * (E - 0.5 * (rhou * rhou) / rho); }
  // :42-45
  double betafun(const V4& U) const {
    double p = pfun(U);
    return U[0] / (2.0 * p);
  }
  // :48-52 (Dim1)
  double wavespeed1(double rho, double rhou, double E) const {
    double p = pfun1(rho, rhou, E);
    return std::fabs(rhou / rho) + std::sqrt(gamma * p / rho);
  }
  // :59-62
  double wavespeed(const V4& U, double n1, double n2) const {
    if (kpp) return 1.0;  // KPP.jl:1-3
    double un = n1 * U[1] + n2 * U[2];
    return wavespeed1(U[0], un, U[3]);
  }
  // :64-68
  double sfun(const V4& U) const {
    double p = pfun(U);
    return std::log(p / std::pow(U[0], gamma));
  }
  // :75-78
  double rhoe_ufun(const V4& U) const { return U[3] - 0.5 * (U[1] * U[1] + U[2] * U[2]) / U[0]; }
  // :93-97
  double s_vfun(const V4& V) const { return gamma - V[0] + (V[1] * V[1] + V[2] * V[2]) / (2.0 * V[3]); }
  // :99-104
  double rhoe_vfun(const V4& V) const {
    double s = s_vfun(V);
    double vE = V[3];
    return std::pow((gamma - 1.0) / std::pow(-vE, gamma), 1.0 / (gamma - 1.0)) * std::exp(-s / (gamma - 1.0));
  }
  // :134-144
  V4 v_ufun(const V4& U) const {
    if (kpp) return U;  // KPP.jl:5-7
    double s = sfun(U);
    double p = pfun(U);
    double v1 = (gamma + 1.0 - s) - (gamma - 1.0) * U[3] / p;
    double vu = U[1] * (gamma - 1.0) / p;
    double vv = U[2] * (gamma - 1.0) / p;
    double vE = -U[0] * (gamma - 1.0) / p;
    return {v1, vu, vv, vE};
  }
  // :155-163
  V4 u_vfun(const V4& V) const {
    if (kpp) return V;  // KPP.jl:9-11
    double rhoeV = rhoe_vfun(V);
    double rho = -rhoeV * V[3];
    double rhou = rhoeV * V[1];
    double rhov = rhoeV * V[2];
    double E = rhoeV * (1.0 - (V[1] * V[1] + V[2] * V[2]) / (2.0 * V[3]));
    return {rho, rhou, rhov, E};
  }
  // :129-132
  std::array<double, 2> psi_ufun(const V4& U) const {
    double gm1 = gamma - 1.0;
    return {gm1 * U[1], gm1 * U[2]};
  }
  // :175-194
  V2x4 fluxes(const V4& U) const {
    if (kpp) {  // KPP.jl:13-18
      V2x4 f;
      f.x = {std::sin(U[0]), 0.0, 0.0, 0.0};
      f.y = {std::cos(U[0]), 0.0, 0.0, 0.0};
      return f;
    }
    double rho = U[0], rhou = U[1], rhov = U[2], E = U[3];
    double p = pfun(U);
    double u = rhou / rho;
    double v = rhov / rho;
    double rhouv = rho * u * v;
    double Ep = E + p;
    V2x4 f;
    f.x = {rhou, rhou * u + p, rhouv, u * Ep};
    f.y = {rhov, rhouv, rhov * v + p, v * Ep};
    return f;
  }
  // :307-321 (coefficients and threshold exactly as the reference)
  static double logmean(double aL, double aR, double logL, double logR) {
    double da = aR - aL;
    double aavg = 0.5 * (aR + aL);
    double f = da / aavg;
    double v = f * f;
    if (std::fabs(f) < 1e-4) {
      return aavg * (1.0 + v * (-0.2 - v * (0.0512 - v * 0.026038857142857)));
    } else {
      return -da / (logL - logR);
    }
  }
  // fS(::KPP{Dim2}) (KPP.jl:25-38) with psi = (-cos u, sin u)
  static V2x4 fS_kpp(double uL, double uR) {
    V2x4 F;
    if (std::fabs(uR - uL) < 1e-12) {
      F.x = {0.5 * (std::sin(uL) + std::sin(uR)), 0.0, 0.0, 0.0};
      F.y = {0.5 * (std::cos(uL) + std::cos(uR)), 0.0, 0.0, 0.0};
    } else {
      F.x = {(-std::cos(uR) - -std::cos(uL)) / (uR - uL), 0.0, 0.0, 0.0};
      F.y = {(std::sin(uR) - std::sin(uL)) / (uR - uL), 0.0, 0.0, 0.0};
    }
    return F;
  }
  // :220-249; UL/UR = (rho, u, v, beta, log rho, log beta)
  V2x4 fS(const double* UL, const double* UR) const {
    double rhoL = UL[0], uL = UL[1], vL = UL[2], betaL = UL[3], rhologL = UL[4], betalogL = UL[5];
    double rhoR = UR[0], uR = UR[1], vR = UR[2], betaR = UR[3], rhologR = UR[4], betalogR = UR[5];
    double rholog = logmean(rhoL, rhoR, rhologL, rhologR);
    double betalog = logmean(betaL, betaR, betalogL, betalogR);
    double rhoavg = 0.5 * (rhoL + rhoR);
    double uavg = 0.5 * (uL + uR);
    double vavg = 0.5 * (vL + vR);
    double unorm = uL * uR + vL * vR;
    double pa = rhoavg / (betaL + betaR);
    double f4aux = rholog / (2.0 * (gamma - 1.0) * betalog) + pa + 0.5 * rholog * unorm;
    double FxS1 = rholog * uavg;
    double FxS2 = FxS1 * uavg + pa;
    double FxS3 = FxS1 * vavg;
    double FxS4 = f4aux * uavg;
    double FyS1 = rholog * vavg;
    double FyS2 = FxS3;
    double FyS3 = FyS1 * vavg + pa;
    double FyS4 = f4aux * vavg;
    V2x4 F;
    F.x = {FxS1, FxS2, FxS3, FxS4};
    F.y = {FyS1, FyS2, FyS3, FyS4};
    return F;
  }
};

// ---------------------------------------------------------------------------
// GLL rule and 1D differentiation matrix (the NodesAndModes/StartUpDG inputs).
// Nodes from Newton iteration on (1-x^2) P_N'(x) written with the Legendre
// recurrence (Hesthaven & Warburton, Nodal DG Methods, JacobiGL/LGL), weights
// 2/(N(N+1) P_N(x_i)^2), D_ij = P_N(x_i)/(P_N(x_j)(x_i-x_j)).
// ---------------------------------------------------------------------------
void gll_rule(int N, std::vector<double>& r, std::vector<double>& w, std::vector<double>& D) {
  int Np = N + 1;
  r.assign(Np, 0.0);
  w.assign(Np, 0.0);
  D.assign(Np * Np, 0.0);
  std::vector<double> x(Np), xold(Np), P(Np * (N + 1));
  for (int i = 0; i < Np; ++i) x[i] = -std::cos(M_PI * i / N);
  auto legendre = [&](const std::vector<double>& xx) {
    for (int i = 0; i < Np; ++i) {
      P[i * (N + 1) + 0] = 1.0;
      if (N >= 1) P[i * (N + 1) + 1] = xx[i];
      for (int k = 2; k <= N; ++k)
        P[i * (N + 1) + k] = ((2.0 * k - 1.0) * xx[i] * P[i * (N + 1) + k - 1] - (k - 1.0) * P[i * (N + 1) + k - 2]) / k;
    }
  };
  for (int it = 0; it < 100; ++it) {
    xold = x;
    legendre(x);
    double err = 0.0;
    for (int i = 0; i < Np; ++i) {
      x[i] = xold[i] - (x[i] * P[i * (N + 1) + N] - P[i * (N + 1) + N - 1]) / (Np * P[i * (N + 1) + N]);
      err = std::max(err, std::fabs(x[i] - xold[i]));
    }
    if (err < 1e-16) break;
  }
  // exact symmetry and endpoints
  for (int i = 0; i < Np / 2; ++i) {
    double a = 0.5 * (x[Np - 1 - i] - x[i]);
    x[i] = -a;
    x[Np - 1 - i] = a;
  }
  if (Np % 2 == 1) x[Np / 2] = 0.0;
  x[0] = -1.0;
  x[Np - 1] = 1.0;
  legendre(x);
  for (int i = 0; i < Np; ++i) {
    double PN = P[i * (N + 1) + N];
    r[i] = x[i];
    w[i] = 2.0 / (N * Np * PN * PN);
  }
  for (int i = 0; i < Np; ++i)
    for (int j = 0; j < Np; ++j) {
      if (i != j) {
        D[i * Np + j] = P[i * (N + 1) + N] / (P[j * (N + 1) + N] * (x[i] - x[j]));
      } else if (i == 0) {
        D[i * Np + j] = -N * (N + 1) / 4.0;
      } else if (i == N) {
        D[i * Np + j] = N * (N + 1) / 4.0;
      } else {
        D[i * Np + j] = 0.0;
      }
    }
}

// ---------------------------------------------------------------------------
// Gauss-Legendre rule (gauss_quad(0, 0, N) of NodesAndModes): the N+1 roots of P_{N+1}
// by Newton iteration from x_i = cos(pi (i + 3/4) / (N + 3/2)), weights
// 2 / ((1 - x^2) P'_{N+1}(x)^2). The Lagrange basis on these nodes in barycentric form
// (Berrut & Trefethen 2004): D_ij = (l_j / l_i) / (x_i - x_j), D_ii = -sum_j D_ij, and
// the values at r = -1, +1 (the face extrapolation of construct_gauss_reference_data,
// init.jl:111-131).
// ---------------------------------------------------------------------------
void gauss_rule(int N, std::vector<double>& r, std::vector<double>& w, std::vector<double>& D,
                std::vector<double>& ell_m1, std::vector<double>& ell_p1) {
  const int n = N + 1;
  r.assign(n, 0.0);
  w.assign(n, 0.0);
  D.assign(n * n, 0.0);
  ell_m1.assign(n, 0.0);
  ell_p1.assign(n, 0.0);
  auto legendre = [&](double x, double& P, double& dP) {  // P_n(x), P_n'(x)
    double p0 = 1.0, p1 = x;
    for (int k = 2; k <= n; ++k) {
      double p2 = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k;
      p0 = p1;
      p1 = p2;
    }
    P = n == 1 ? x : p1;
    if (n == 1) p0 = 1.0;
    dP = n * (x * P - p0) / (x * x - 1.0);
  };
  for (int i = 0; i < n; ++i) {
    double x = -std::cos(3.141592653589793 * (i + 0.75) / (n + 0.5));
    for (int it = 0; it < 100; ++it) {
      double P, dP;
      legendre(x, P, dP);
      double dx = P / dP;
      x -= dx;
      if (std::fabs(dx) < 1e-16) break;
    }
    r[i] = x;
  }
  for (int i = 0; i < n / 2; ++i) {  // exact symmetry
    double a = 0.5 * (r[n - 1 - i] - r[i]);
    r[i] = -a;
    r[n - 1 - i] = a;
  }
  if (n % 2 == 1) r[n / 2] = 0.0;
  for (int i = 0; i < n; ++i) {
    double P, dP;
    legendre(r[i], P, dP);
    w[i] = 2.0 / ((1.0 - r[i] * r[i]) * dP * dP);
  }
  std::vector<double> lam(n, 1.0);
  for (int j = 0; j < n; ++j)
    for (int k = 0; k < n; ++k)
      if (k != j) lam[j] /= (r[j] - r[k]);
  for (int i = 0; i < n; ++i) {
    double diag = 0.0;
    for (int j = 0; j < n; ++j)
      if (j != i) {
        D[i * n + j] = (lam[j] / lam[i]) / (r[i] - r[j]);
        diag -= D[i * n + j];
      }
    D[i * n + i] = diag;
  }
  for (int side = 0; side < 2; ++side) {
    const double x = side == 0 ? -1.0 : 1.0;
    double den = 0.0;
    for (int j = 0; j < n; ++j) den += lam[j] / (x - r[j]);
    for (int j = 0; j < n; ++j) (side == 0 ? ell_m1 : ell_p1)[j] = (lam[j] / (x - r[j])) / den;
  }
}

struct Solver {
  // sizes (SizeData, Solver.jl:173-183)
  int N, N1D, Nq, Nfp, Nh, K, Ns = 3;
  // CompressibleEulerIdealGas{Dim1}: Nd = 1, Nq = N1D, Nfp = 2; states keep four slots with
  // the y momentum 0, so every Dim2 point function gives the Dim1 value exactly
  bool dim1 = false;
  int Nd = 2;
  p2de_param prm;
  Euler eq;
  int nthreads = 1;
  std::string err;

  // operators (Operators, Solver.jl:192-212), column-major dense like the reference
  std::vector<double> r1D, w1D, D1D, wq;
  std::vector<double> Srh_db, Ssh_db;  // Nh x Nh
  std::vector<double> Sr0, Ss0;        // Nq x Nq
  std::vector<double> Br, Bs;          // Nfp diagonal entries
  std::vector<double> Vf, Vf_low;      // Nfp x Nq
  std::vector<double> MinvVhT;         // Nq x Nh
  std::vector<double> MinvVfT;         // Nq x Nfp
  std::vector<std::pair<int, int>> Srsh_nnz, Srs0_nnz;  // 0-based (i, j)
  std::vector<int> fq2q;
  std::vector<std::vector<int>> q2fq;

  // geometry (GeomData): Jq (Nq x K), GJh = rxJh, sxJh, ryJh, syJh (Nh x K)
  std::vector<double> Jq, rxJh, sxJh, ryJh, syJh;

  // BCData (StateParam.jl:1-7) plus the wall / moving-shock extension
  std::vector<int64_t> mapP, mapI, mapO, mapW, mapS;
  std::vector<V4> Ival;
  std::vector<double> xyS;
  double shock_x0 = 0, shock_inv_slope = 0, shock_speed = 0;
  V4 shock_post{}, shock_pre{};

  // Preallocation (State.jl:1-26)
  std::vector<V4> Uq, vq, u_tilde, v_tilde, rhsH, rhsL, rhsU, resW, resZ;
  std::vector<std::array<double, 2>> psi_tilde;
  std::vector<V2x4> rhsxyH, rhsxyL, rhsxyU, BF_H, BF_L, fstar_H, fstar_L;
  std::vector<double> L_local;  // (Nq+N1D) x 2 x K x Ns

  // LowOrderPositivityCache (State.jl:29-50)
  std::vector<V2x4> flux, Q0F1;
  std::vector<double> wavespeed_f, lambda, lambdaB;
  std::vector<V4> Uf, uP_L;
  // FluxDiffCache (State.jl:52-85)
  std::vector<double> beta, rholog, betalog, betaP, rhologP, betalogP, lam, LFc;
  std::vector<V4> uP_H;
  std::vector<V2x4> QF1, MinvVhTQF1, MinvVfTBF1;
  // SubcellLimiterCache (State.jl:131-185)
  std::vector<V4> f_bar_H[2], f_bar_L[2], f_bar_lim[2], vf;
  std::vector<std::array<double, 2>> psif, sum_Bpsi, sum_dvfbarL;
  std::vector<double> dvdf[2];

  // ---- index helpers (0-based) ----
  size_t LL(int i, int d, int k, int s) const { return (size_t)i + (size_t)(Nq + N1D) * (d + Nd * ((size_t)k + (size_t)K * s)); }
  void face_of(int64_t m1, int& iP, int& kP) const {  // mapP value (1-based) -> (face node, element)
    iP = (int)((m1 - 1) % Nfp);
    kP = (int)((m1 - 1) / Nfp);
  }

  // rhs_utils.jl:340-344
  static std::array<double, 2> reference_to_physical(double Ur, double Us, double rxJ, double sxJ, double ryJ, double syJ) {
    return {rxJ * Ur + sxJ * Us, ryJ * Ur + syJ * Us};
  }
  // LinearAlgebra generic norm2 of a 2-tuple (no rescaling needed for finite data)
  static double norm2(double a, double b) {
    double m = std::max(std::fabs(a), std::fabs(b));
    if (m == 0.0 || std::isinf(m) || std::isnan(m)) return m;
    return std::sqrt(a * a + b * b);
  }
  // rhs_utils.jl:354-360
  std::array<double, 2> Bx(int f, int k) const {
    size_t h = (size_t)(Nq + f) + (size_t)Nh * k;
    return reference_to_physical(Br[f], Bs[f], rxJh[h], sxJh[h], ryJh[h], syJh[h]);
  }
  // rhs_utils.jl:379-384
  std::array<double, 2> Sx(int i, int j, int k) const {
    size_t h = (size_t)i + (size_t)Nh * k;
    return reference_to_physical(Srh_db[i + (size_t)Nh * j], Ssh_db[i + (size_t)Nh * j], rxJh[h], sxJh[h], ryJh[h], syJh[h]);
  }
  // rhs_utils.jl:393-398
  std::array<double, 2> Sx0(int i, int j, int k) const {
    size_t h = (size_t)i + (size_t)Nh * k;
    return reference_to_physical(Sr0[i + (size_t)Nq * j], Ss0[i + (size_t)Nq * j], rxJh[h], sxJh[h], ryJh[h], syJh[h]);
  }

  // ---------------------------------------------------------------------------
  // initialize_operators (init.jl:133-228) for LGL quads (init.jl:97-103, 307-340)
  // ---------------------------------------------------------------------------
  // inv(VDM) (init.jl:224) for LGL: VDM = vandermonde(Quad(), N, r, s) of NodesAndModes,
  // the orthonormal Legendre products P_i(r) P_j(s) (mode i + N1D j) at the nodes
  std::vector<double> VDMinv;  // Nq x Nq, row-major
  static double legendre_orthonormal(int n, double x) {
    double p0 = 1.0, p1 = x;
    if (n == 0) return std::sqrt(0.5);
    for (int k = 1; k < n; ++k) {
      double p2 = ((2.0 * k + 1.0) * x * p1 - k * p0) / (k + 1.0);
      p0 = p1;
      p1 = p2;
    }
    return std::sqrt((2.0 * n + 1.0) / 2.0) * p1;
  }
  void build_vdm_inv() {
    std::vector<double> A((size_t)Nq * Nq), Inv((size_t)Nq * Nq, 0.0);
    if (dim1) {  // Line: P_j(r_i), mode j
      for (int i = 0; i < N1D; ++i)
        for (int j = 0; j < N1D; ++j) A[(size_t)i * Nq + j] = legendre_orthonormal(j, r1D[i]);
    } else {
      for (int is = 0; is < N1D; ++is)
        for (int ir = 0; ir < N1D; ++ir)
          for (int j = 0; j < N1D; ++j)
            for (int i = 0; i < N1D; ++i)
              A[(size_t)(ir + N1D * is) * Nq + (i + N1D * j)] = legendre_orthonormal(i, r1D[ir]) * legendre_orthonormal(j, r1D[is]);
    }
    for (int i = 0; i < Nq; ++i) Inv[(size_t)i * Nq + i] = 1.0;
    // Gauss-Jordan elimination with partial pivoting
    for (int c = 0; c < Nq; ++c) {
      int piv = c;
      for (int r = c + 1; r < Nq; ++r)
        if (std::fabs(A[(size_t)r * Nq + c]) > std::fabs(A[(size_t)piv * Nq + c])) piv = r;
      if (piv != c)
        for (int j = 0; j < Nq; ++j) {
          std::swap(A[(size_t)c * Nq + j], A[(size_t)piv * Nq + j]);
          std::swap(Inv[(size_t)c * Nq + j], Inv[(size_t)piv * Nq + j]);
        }
      const double d = A[(size_t)c * Nq + c];
      for (int j = 0; j < Nq; ++j) {
        A[(size_t)c * Nq + j] /= d;
        Inv[(size_t)c * Nq + j] /= d;
      }
      for (int r = 0; r < Nq; ++r) {
        if (r == c) continue;
        const double f = A[(size_t)r * Nq + c];
        if (f == 0.0) continue;
        for (int j = 0; j < Nq; ++j) {
          A[(size_t)r * Nq + j] -= f * A[(size_t)c * Nq + j];
          Inv[(size_t)r * Nq + j] -= f * Inv[(size_t)c * Nq + j];
        }
      }
    }
    VDMinv = Inv;
  }

  // initialize_smoothness_indicator!(::Dim2) (shock_capture.jl:47-81, 92-103): per
  // element, the modal energies of rho*p through inv(VDM); smooth_indicator =
  // max(E_N, E_{N-1}) / E. update_blending_factor! (HennemannShockCapture, :118-137):
  // max(min(1 - alpha, 1), 1/2). update_smoothness_factor! (subcell.jl:927-956): 0 for
  // the plain positivity/TVD/cell-entropy bounds, 1 for the min-entropy bounds, and for
  // the relaxed bounds 0 / 1 / 1/2 - 1/2 sin(pi (s_k - s_0) / 2) with s_k the log10 of
  // the indicator, s_0 = log10(N^-4) and kappa = 1.
  std::vector<double> blending_factor, smooth_indicator, smooth_factor;
  void update_smoothness() {
    smooth_indicator.assign(K, 0.0);
#pragma omp parallel for schedule(static)
    for (int k = 0; k < K; ++k) {
      std::vector<double> ind(Nq), modal(Nq);
      for (int i = 0; i < Nq; ++i) {
        const V4& U = Uq[i + (size_t)Nq * k];
        ind[i] = eq.kpp ? U[0] : U[0] * eq.pfun(U);  // initialize_indicator! (shock_capture.jl:83-105)
      }
      for (int i = 0; i < Nq; ++i) {
        double sum = 0.0;
        for (int j = 0; j < Nq; ++j) sum += VDMinv[(size_t)i * Nq + j] * ind[j];
        modal[i] = sum;
      }
      double modeN = 0.0, modeNm1 = 0.0, total = 0.0;
      int count = 0;
      for (int j = 0; j <= (dim1 ? 0 : N); ++j)  // initialize_smoothness_indicator!(::Dim1) (shock_capture.jl:14-45): modes i
        for (int i = 0; i <= N; ++i) {
          const double energy = modal[count] * modal[count];
          if (i == N || (!dim1 && j == N)) modeN += energy;
          if (i == N - 1 || (!dim1 && j == N - 1)) modeNm1 += energy;
          total += energy;
          ++count;
        }
      smooth_indicator[k] = jmax(modeN / total, modeNm1 / total);
    }
    blending_factor.assign(K, 1.0);
    if (prm.shock_capture == 1) {
      const double a = prm.shock_capture_a, c = prm.shock_capture_c;
      const double TN = a * std::pow(10.0, -c * std::pow((double)(N + 1), 0.25));
      const double alphamax = 0.5, alphaE0 = 0.0001;
      const double s_factor = std::log((1 - alphaE0) / alphaE0);
      for (int k = 0; k < K; ++k) {
        const double alpha = 1.0 / (1.0 + std::exp(-s_factor / TN * (smooth_indicator[k] - TN)));
        blending_factor[k] = jmax(jmin(1.0 - alpha, 1.0), alphamax);
      }
    }
    smooth_factor.assign(K, min_entropy() && !relaxed() ? 1.0 : 0.0);
    if (relaxed()) {
      const double kappa = 1.0;
      const double s0 = std::log(1.0 / ((double)N * N * N * N)) / std::log(10.0);
      for (int k = 0; k < K; ++k) {
        const double sk = std::log(smooth_indicator[k]) / std::log(10.0);
        if (sk < s0 - kappa) smooth_factor[k] = 0.0;
        else if (sk > s0 + kappa) smooth_factor[k] = 1.0;
        else smooth_factor[k] = 0.5 - 0.5 * std::sin(3.141592653589793 * (sk - s0) / (2 * kappa));
      }
    }
  }

  void build_operators() {
    if (dim1) {
      build_operators_1d();
      return;
    }
    N1D = N + 1;
    Nq = N1D * N1D;
    Nfp = 4 * N1D;
    Nh = Nq + Nfp;
    std::vector<double> ell_m1, ell_p1;  // Lagrange basis at r = -1, +1 (Gauss)
    if (gauss())
      gauss_rule(N, r1D, w1D, D1D, ell_m1, ell_p1);
    else
      gll_rule(N, r1D, w1D, D1D);
    build_vdm_inv();
    const double ZEROTOL = prm.ZEROTOL;
    // tensor-product nodes, r fastest: i = ir + N1D*is
    wq.assign(Nq, 0.0);
    for (int is = 0; is < N1D; ++is)
      for (int ir = 0; ir < N1D; ++ir) wq[ir + N1D * is] = w1D[ir] * w1D[is];
    // Dr = kron(I, D1D), Ds = kron(D1D, I); Qrs = Pq'*M*Drs*Pq with M = diag(wq), Pq = I (init.jl:149)
    std::vector<double> Qr(Nq * Nq, 0.0), Qs(Nq * Nq, 0.0);  // column-major
    for (int is = 0; is < N1D; ++is)
      for (int ir = 0; ir < N1D; ++ir)
        for (int jr = 0; jr < N1D; ++jr) {
          int i = ir + N1D * is, j = jr + N1D * is;
          Qr[i + Nq * j] = wq[i] * D1D[ir * N1D + jr];
        }
    for (int ir = 0; ir < N1D; ++ir)
      for (int is = 0; is < N1D; ++is)
        for (int js = 0; js < N1D; ++js) {
          int i = ir + N1D * is, j = ir + N1D * js;
          Qs[i + Nq * j] = wq[i] * D1D[is * N1D + js];
        }
    for (auto& q : Qr)
      if (std::fabs(q) <= ZEROTOL) q = 0.0;  // droptol!
    for (auto& q : Qs)
      if (std::fabs(q) <= ZEROTOL) q = 0.0;
    // faces: r=-1, r=+1, s=-1, s=+1; nrJ, nsJ; wf = repeat(w1D, 4)
    fq2q.assign(Nfp, 0);
    Br.assign(Nfp, 0.0);
    Bs.assign(Nfp, 0.0);
    for (int j = 0; j < N1D; ++j) {
      fq2q[j] = 0 + N1D * j;
      fq2q[N1D + j] = N + N1D * j;
      fq2q[2 * N1D + j] = j;
      fq2q[3 * N1D + j] = j + N1D * N;
      Br[j] = w1D[j] * -1.0;
      Br[N1D + j] = w1D[j] * 1.0;
      Bs[2 * N1D + j] = w1D[j] * -1.0;
      Bs[3 * N1D + j] = w1D[j] * 1.0;
    }
    // Vf_low: the face node's nearest volume node (init.jl:324-340); for LGL it is also Vf
    // (a selection matrix; init.jl:180-185 rounds its near-one entries to one). Gauss:
    // Vf extrapolates along the line normal to the face, Vf[f, i] = l_a(-1 or +1) for the
    // node a of that line (construct_gauss_reference_data, init.jl:111-131).
    Vf.assign(Nfp * Nq, 0.0);
    for (int f = 0; f < Nfp; ++f) Vf[f + (size_t)Nfp * fq2q[f]] = 1.0;
    Vf_low = Vf;
    if (gauss()) {
      std::fill(Vf.begin(), Vf.end(), 0.0);
      for (int f = 0; f < Nfp; ++f) {
        const int side = f / N1D, t = f % N1D;
        const std::vector<double>& ell = (side % 2 == 0) ? ell_m1 : ell_p1;
        for (int a = 0; a < N1D; ++a) {
          const int i = side < 2 ? a + N1D * t : t + N1D * a;
          Vf[f + (size_t)Nfp * i] = std::fabs(ell[a]) <= ZEROTOL ? 0.0 : ell[a];
        }
      }
    }
    // hybridized SBP (init.jl:152-155): Srsh_db = [Q-Q', Ef'B; -B Ef, 0], Ef = Vf Pq = Vf
    Srh_db.assign((size_t)Nh * Nh, 0.0);
    Ssh_db.assign((size_t)Nh * Nh, 0.0);
    for (int j = 0; j < Nq; ++j)
      for (int i = 0; i < Nq; ++i) {
        Srh_db[i + (size_t)Nh * j] = Qr[i + Nq * j] - Qr[j + Nq * i];
        Ssh_db[i + (size_t)Nh * j] = Qs[i + Nq * j] - Qs[j + Nq * i];
      }
    for (int f = 0; f < Nfp; ++f)
      for (int i = 0; i < Nq; ++i) {
        const double e = Vf[f + (size_t)Nfp * i];
        if (e == 0.0) continue;
        Srh_db[i + (size_t)Nh * (Nq + f)] = e * Br[f];
        Ssh_db[i + (size_t)Nh * (Nq + f)] = e * Bs[f];
        Srh_db[(Nq + f) + (size_t)Nh * i] = -(Br[f] * e);
        Ssh_db[(Nq + f) + (size_t)Nh * i] = -(Bs[f] * e);
      }
    if (gauss()) {  // droptol! of the hybridized 0.5 [...] (init.jl:152-154)
      for (auto& q : Srh_db)
        if (std::fabs(0.5 * q) <= ZEROTOL) q = 0.0;
      for (auto& q : Ssh_db)
        if (std::fabs(0.5 * q) <= ZEROTOL) q = 0.0;
    }
    // MinvVhT = M \ Vh', MinvVfT = M \ Vf' (init.jl:171-172), M = diag(wq)
    MinvVhT.assign((size_t)Nq * Nh, 0.0);
    MinvVfT.assign((size_t)Nq * Nfp, 0.0);
    for (int i = 0; i < Nq; ++i) MinvVhT[i + (size_t)Nq * i] = 1.0 / wq[i];
    for (int f = 0; f < Nfp; ++f)
      for (int i = 0; i < Nq; ++i) {
        const double e = Vf[f + (size_t)Nfp * i];
        if (e == 0.0) continue;
        MinvVhT[i + (size_t)Nq * (Nq + f)] = e / wq[i];
        MinvVfT[i + (size_t)Nq * f] = e / wq[i];
      }
    // low order operators (init.jl:276-295, 312-322): Q01D tridiagonal, Sr0 = 0.5(Qr0-Qr0')
    std::vector<double> Q01D(N1D * N1D, 0.0);  // column-major
    for (int i = 0; i < N1D; ++i) {
      if (i + 1 < N1D) {
        Q01D[(i + 1) + N1D * i] = -0.5;  // dl
        Q01D[i + N1D * (i + 1)] = 0.5;   // du
      }
    }
    Q01D[0] = -0.5;
    Q01D[(N1D - 1) + N1D * (N1D - 1)] = 0.5;
    Sr0.assign(Nq * Nq, 0.0);
    Ss0.assign(Nq * Nq, 0.0);
    std::vector<double> Qr0(Nq * Nq, 0.0), Qs0(Nq * Nq, 0.0);
    for (int is = 0; is < N1D; ++is)
      for (int js = 0; js < N1D; ++js)
        for (int ir = 0; ir < N1D; ++ir)
          for (int jr = 0; jr < N1D; ++jr) {
            int i = ir + N1D * is, j = jr + N1D * js;
            double M1Dss = (is == js) ? w1D[is] : 0.0;
            double M1Drr = (ir == jr) ? w1D[ir] : 0.0;
            Qr0[i + Nq * j] = M1Dss * Q01D[ir + N1D * jr];  // kron(M1D, Q01D)
            Qs0[i + Nq * j] = Q01D[is + N1D * js] * M1Drr;  // kron(Q01D, M1D)
          }
    for (int j = 0; j < Nq; ++j)
      for (int i = 0; i < Nq; ++i) {
        double a = 0.5 * (Qr0[i + Nq * j] - Qr0[j + Nq * i]);
        double b = 0.5 * (Qs0[i + Nq * j] - Qs0[j + Nq * i]);
        Sr0[i + Nq * j] = std::fabs(a) <= ZEROTOL ? 0.0 : a;
        Ss0[i + Nq * j] = std::fabs(b) <= ZEROTOL ? 0.0 : b;
      }
    // nnz lists (init.jl:188-204): j outer, i = j+1.. inner
    Srsh_nnz.clear();
    for (int j = 0; j < Nh; ++j)
      for (int i = j + 1; i < Nh; ++i)
        if (std::fabs(Srh_db[i + (size_t)Nh * j]) + std::fabs(Ssh_db[i + (size_t)Nh * j]) != 0.0) Srsh_nnz.push_back({i, j});
    Srs0_nnz.clear();
    for (int j = 0; j < Nq; ++j)
      for (int i = j + 1; i < Nq; ++i)
        if (std::fabs(Sr0[i + Nq * j]) + std::fabs(Ss0[i + Nq * j]) != 0.0) Srs0_nnz.push_back({i, j});
    // q2fq (init.jl:215-220): ascending face index
    q2fq.assign(Nq, {});
    for (int i = 0; i < Nq; ++i)
      for (int f = 0; f < Nfp; ++f)
        if (Vf_low[f + (size_t)Nfp * i] == 1.0) q2fq[i].push_back(f);
  }

  // initialize_reference_data(::Dim1) (init.jl:66-80) and initialize_operators (:133-228) on
  // a Line: LGL or Gauss nodes (Gauss through construct_gauss_reference_data, :83-131), faces
  // r = -1, +1 with nrJ = -1, +1 and wf = 1, and the low-order Sr0 = (Q0 - Q0')/2 of the
  // tridiagonal Q0 (construct_low_order_operators_1D, :276-301; no mass weights on a Line).
  // On LGL nodes Vq and Vf are taken as the exact identity and selection, where the
  // reference's Vandermonde products carry rounding of about 1e-16.
  void build_operators_1d() {
    N1D = N + 1;
    Nq = N1D;
    Nfp = 2;
    Nh = Nq + Nfp;
    std::vector<double> ell_m1, ell_p1;
    if (gauss())
      gauss_rule(N, r1D, w1D, D1D, ell_m1, ell_p1);
    else
      gll_rule(N, r1D, w1D, D1D);
    build_vdm_inv();
    const double ZEROTOL = prm.ZEROTOL;
    wq = w1D;
    std::vector<double> Qr(Nq * Nq, 0.0);  // M Dr, column-major
    for (int i = 0; i < Nq; ++i)
      for (int j = 0; j < Nq; ++j) {
        const double q = wq[i] * D1D[i * N1D + j];
        Qr[i + Nq * j] = std::fabs(q) <= ZEROTOL ? 0.0 : q;
      }
    fq2q = {0, N};
    Br = {-1.0, 1.0};
    Bs = {0.0, 0.0};
    Vf.assign(Nfp * Nq, 0.0);
    Vf[0 + (size_t)Nfp * 0] = 1.0;
    Vf[1 + (size_t)Nfp * N] = 1.0;
    Vf_low = Vf;
    if (gauss())
      for (int i = 0; i < Nq; ++i) {
        Vf[0 + (size_t)Nfp * i] = std::fabs(ell_m1[i]) <= ZEROTOL ? 0.0 : ell_m1[i];
        Vf[1 + (size_t)Nfp * i] = std::fabs(ell_p1[i]) <= ZEROTOL ? 0.0 : ell_p1[i];
      }
    // Srh_db = [Q - Q', Ef' B; -B Ef, 0] (init.jl:152-155)
    Srh_db.assign((size_t)Nh * Nh, 0.0);
    Ssh_db.assign((size_t)Nh * Nh, 0.0);
    for (int j = 0; j < Nq; ++j)
      for (int i = 0; i < Nq; ++i) Srh_db[i + (size_t)Nh * j] = Qr[i + Nq * j] - Qr[j + Nq * i];
    for (int f = 0; f < Nfp; ++f)
      for (int i = 0; i < Nq; ++i) {
        const double e = Vf[f + (size_t)Nfp * i];
        if (e == 0.0) continue;
        Srh_db[i + (size_t)Nh * (Nq + f)] = e * Br[f];
        Srh_db[(Nq + f) + (size_t)Nh * i] = -(Br[f] * e);
      }
    if (gauss())
      for (auto& q : Srh_db)
        if (std::fabs(0.5 * q) <= ZEROTOL) q = 0.0;
    MinvVhT.assign((size_t)Nq * Nh, 0.0);
    MinvVfT.assign((size_t)Nq * Nfp, 0.0);
    for (int i = 0; i < Nq; ++i) MinvVhT[i + (size_t)Nq * i] = 1.0 / wq[i];
    for (int f = 0; f < Nfp; ++f)
      for (int i = 0; i < Nq; ++i) {
        const double e = Vf[f + (size_t)Nfp * i];
        if (e == 0.0) continue;
        MinvVhT[i + (size_t)Nq * (Nq + f)] = e / wq[i];
        MinvVfT[i + (size_t)Nq * f] = e / wq[i];
      }
    // Q0: d = (-1/2, 0, ..., 0, 1/2), dl = -1/2, du = 1/2; Sr0 = (Q0 - Q0')/2
    Sr0.assign(Nq * Nq, 0.0);
    Ss0.assign(Nq * Nq, 0.0);
    for (int i = 0; i + 1 < Nq; ++i) {
      Sr0[i + Nq * (i + 1)] = 0.5 * (0.5 - -0.5);
      Sr0[(i + 1) + Nq * i] = 0.5 * (-0.5 - 0.5);
    }
    Srsh_nnz.clear();
    for (int j = 0; j < Nh; ++j)
      for (int i = j + 1; i < Nh; ++i)
        if (std::fabs(Srh_db[i + (size_t)Nh * j]) != 0.0) Srsh_nnz.push_back({i, j});
    Srs0_nnz.clear();
    for (int j = 0; j < Nq; ++j)
      for (int i = j + 1; i < Nq; ++i)
        if (std::fabs(Sr0[i + Nq * j]) != 0.0) Srs0_nnz.push_back({i, j});
    q2fq.assign(Nq, {});
    q2fq[0].push_back(0);
    q2fq[N].push_back(1);
  }

  void allocate() {
    size_t nq = (size_t)Nq * K, nh = (size_t)Nh * K, nf = (size_t)Nfp * K;
    Uq.assign(nq, V4{});
    vq.assign(nq, V4{});
    u_tilde.assign(nh, V4{});
    v_tilde.assign(nh, V4{});
    psi_tilde.assign(nh, {0.0, 0.0});
    rhsH.assign(nq, V4{});
    rhsL.assign(nq, V4{});
    rhsU.assign(nq, V4{});
    resW.assign(nq, V4{});
    resZ.assign(nq, V4{});
    rhsxyH.assign(nq, V2x4{});
    rhsxyL.assign(nq, V2x4{});
    rhsxyU.assign(nq, V2x4{});
    BF_H.assign(nf, V2x4{});
    BF_L.assign(nf, V2x4{});
    fstar_H.assign(nf, V2x4{});
    fstar_L.assign(nf, V2x4{});
    L_local.assign((size_t)(Nq + N1D) * Nd * K * Ns, 0.0);
    L_elem.assign((size_t)K * Ns, 0.0);
    theta_local.assign((size_t)Nfp * K * Ns, 1.0);
    flux.assign(nh, V2x4{});
    Q0F1.assign(nq, V2x4{});
    wavespeed_f.assign(nf, 0.0);
    lambda.assign((size_t)Nq * Nq * K, 0.0);
    lambdaB.assign(nf, 0.0);
    Uf.assign(nf, V4{});
    uP_L.assign(nf, V4{});
    beta.assign(nh, 0.0);
    rholog.assign(nh, 0.0);
    betalog.assign(nh, 0.0);
    betaP.assign(nf, 0.0);
    rhologP.assign(nf, 0.0);
    betalogP.assign(nf, 0.0);
    lam.assign(nf, 0.0);
    LFc.assign(nf, 0.0);
    uP_H.assign(nf, V4{});
    QF1.assign(nh, V2x4{});
    MinvVhTQF1.assign(nq, V2x4{});
    MinvVfTBF1.assign(nq, V2x4{});
    for (int d = 0; d < 2; ++d) {
      f_bar_H[d].assign((size_t)(Nq + N1D) * K, V4{});
      f_bar_L[d].assign((size_t)(Nq + N1D) * K, V4{});
      f_bar_lim[d].assign((size_t)(Nq + N1D) * K, V4{});
      dvdf[d].assign((size_t)(dim1 ? N1D - 1 : Nq - N1D) * K, 0.0);
    }
    vf.assign(nf, V4{});
    psif.assign(nf, {0.0, 0.0});
    sum_Bpsi.assign(K, {0.0, 0.0});
    sum_dvfbarL.assign(K, {0.0, 0.0});
  }

  // state at a moving-shock boundary node (extension; no BCData counterpart)
  V4 shock_state(int64_t idx, double t) const {
    double x = xyS[2 * idx], y = xyS[2 * idx + 1];
    return (x < shock_x0 + (y + shock_speed * t) * shock_inv_slope) ? shock_post : shock_pre;
  }
  static V4 reflect(const V4& U, double n1, double n2) {
    double mn = U[1] * n1 + U[2] * n2;
    return {U[0], U[1] - 2.0 * mn * n1, U[2] - 2.0 * mn * n2, U[3]};
  }
  std::array<double, 2> unit_normal(int64_t lin) const {
    int f = (int)(lin % Nfp), k = (int)(lin / Nfp);
    auto B = Bx(f, k);
    double nn = norm2(B[0], B[1]);
    return {B[0] / nn, B[1] / nn};
  }

  // ---------------------------------------------------------------------------
  // entropy_projection!(::NoEntropyProjectionLimiter) (rhs.jl:217-268)
  // ---------------------------------------------------------------------------
  // entropy_projection! (rhs.jl:59-133): volume nodes keep Uq; face node f takes
  // u(sum_j (theta Vf[f,j] + (1 - theta) Vf_low[f,j]) v(Uq_j)), theta = 1 without the
  // limiter (entropy_projection_face_node!, :87-95)
  std::vector<double> theta_local;  // Nfp x K x Ns
  V4 face_entropy_var(int f, int k, double th) const {
    V4 acc{0.0, 0.0, 0.0, 0.0};
    for (int j = 0; j < Nq; ++j) {
      double c = th * Vf[f + (size_t)Nfp * j] + (1.0 - th) * Vf_low[f + (size_t)Nfp * j];
      acc = add(acc, scal(c, vq[j + (size_t)Nq * k]));
    }
    return acc;
  }
  void entropy_projection(int nstage) {
    const int s = nstage - 1;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < K; ++k) {
      for (int i = 0; i < Nq; ++i) vq[i + (size_t)Nq * k] = eq.v_ufun(Uq[i + (size_t)Nq * k]);
      for (int i = 0; i < Nq; ++i) {
        v_tilde[i + (size_t)Nh * k] = vq[i + (size_t)Nq * k];
        u_tilde[i + (size_t)Nh * k] = Uq[i + (size_t)Nq * k];
      }
      for (int f = 0; f < Nfp; ++f) {
        const double l = scaled_extrapolation() ? theta_local[f + (size_t)Nfp * (k + (size_t)K * s)] : 1.0;
        V4 acc = face_entropy_var(f, k, l);
        v_tilde[Nq + f + (size_t)Nh * k] = acc;
        u_tilde[Nq + f + (size_t)Nh * k] = eq.u_vfun(acc);
      }
    }
  }

  // compute_entropyproj_limiting_param!(::GaussCollocation) (filter.jl:6-16),
  // calc_face_values! (:28-46), solve_theta!(::NodewiseScaledExtrapolation) (:53-62):
  // per face node the largest theta on the bisection grid of [0, 1] whose face value is
  // well defined (vE < -POSTOL) and inside the bounds of check_bound_on_face_node (:91-102)
  void solve_theta(int nstage) {
    const int s = nstage - 1;
    const double eps = prm.POSTOL, zeta = prm.zeta, eta = prm.eta;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < K; ++k) {
      for (int i = 0; i < Nq; ++i) vq[i + (size_t)Nq * k] = eq.v_ufun(Uq[i + (size_t)Nq * k]);
      for (int f = 0; f < Nfp; ++f) {
        V4 Ufv{0.0, 0.0, 0.0, 0.0}, VUf{0.0, 0.0, 0.0, 0.0};
        for (int j = 0; j < Nq; ++j) {
          Ufv = add(Ufv, scal(Vf[f + (size_t)Nfp * j], Uq[j + (size_t)Nq * k]));
          VUf = add(VUf, scal(Vf[f + (size_t)Nfp * j], vq[j + (size_t)Nq * k]));
        }
        const double rhoef = eq.rhoe_ufun(Ufv);
        auto ok = [&](double th) {
          V4 vt = face_entropy_var(f, k, th);
          if (!(vt[3] < -eps)) return false;  // update_limited_entropyproj_vars_on_face_node! (:111-130)
          V4 ut = eq.u_vfun(vt);
          const double v3 = vt[3], rho = ut[0], rhoe = eq.rhoe_ufun(ut);
          return v3 < jmin(zeta * VUf[3], -eps) && rho > jmax((1 - eta) * Ufv[0], eps) &&
                 rho < (1 + eta) * Ufv[0] && rhoe > jmax((1 - eta) * rhoef, eps) && rhoe < (1 + eta) * rhoef;
        };
        // bisection(f, 0.0, 1.0) (nonlinear_solvers.jl:3-20)
        double x_valid = 0.0, x_invalid = 1.0, th;
        if (ok(x_invalid)) {
          th = x_invalid;
        } else {
          for (int iter = 0; iter <= 20; ++iter) {
            const double x_new = 0.5 * (x_valid + x_invalid);
            if (ok(x_new)) x_valid = x_new;
            else x_invalid = x_new;
          }
          th = x_valid;
        }
        theta_local[f + (size_t)Nfp * (k + (size_t)K * s)] = th;
      }
    }
  }

  // ---------------------------------------------------------------------------
  // rhs_low_graph_visc! (low_order_graph_viscosity.jl:4-41)
  // ---------------------------------------------------------------------------
  double rhs_low_graph_visc(double t, double dt, int nstage) {
    // calculate_wavespeed_and_inviscid_flux! (:43-92): face values by update_face_values!,
    // LaxFriedrichsOnNodalVal (:51-61) or LaxFriedrichsOnProjectedVal (:63-71)
    const bool lf_proj = prm.low_order_surface_flux == P2DE_FLUX_LAX_FRIEDRICHS_ON_PROJECTED_VAL;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < K; ++k) {
      for (int f = 0; f < Nfp; ++f)
        Uf[f + (size_t)Nfp * k] = lf_proj ? u_tilde[Nq + f + (size_t)Nh * k] : Uq[fq2q[f] + (size_t)Nq * k];
      for (int i = 0; i < Nq; ++i) flux[i + (size_t)Nh * k] = eq.fluxes(Uq[i + (size_t)Nq * k]);
      for (int f = 0; f < Nfp; ++f) {
        const V4& u = Uf[f + (size_t)Nfp * k];
        auto B = Bx(f, k);
        double nn = norm2(B[0], B[1]);
        wavespeed_f[f + (size_t)Nfp * k] = eq.wavespeed(u, B[0] / nn, B[1] / nn);
        flux[Nq + f + (size_t)Nh * k] = eq.fluxes(u);
      }
    }
    // get_uP_and_enforce_BC! (:94-124)
#pragma omp parallel for schedule(static)
    for (int k = 0; k < K; ++k)
      for (int f = 0; f < Nfp; ++f) {
        int iP, kP;
        face_of(mapP[f + (size_t)Nfp * k], iP, kP);
        uP_L[f + (size_t)Nfp * k] = Uf[iP + (size_t)Nfp * kP];
      }
    for (size_t i = 0; i < mapI.size(); ++i) uP_L[mapI[i] - 1] = Ival[i];
    for (size_t i = 0; i < mapO.size(); ++i) {
      int iP, kP;
      face_of(mapO[i], iP, kP);
      uP_L[mapO[i] - 1] = Uq[fq2q[iP] + (size_t)Nq * kP];
    }
    for (size_t i = 0; i < mapW.size(); ++i) {
      auto n = unit_normal(mapW[i] - 1);
      uP_L[mapW[i] - 1] = reflect(Uf[mapW[i] - 1], n[0], n[1]);
    }
    for (size_t i = 0; i < mapS.size(); ++i) uP_L[mapS[i] - 1] = shock_state((int64_t)i, t);
    // clear_low_order_rhs! (:126-137)
#pragma omp parallel for schedule(static)
    for (int k = 0; k < K; ++k)
      for (int i = 0; i < Nq; ++i) {
        rhsxyL[i + (size_t)Nq * k] = V2x4{};
        Q0F1[i + (size_t)Nq * k] = V2x4{};
      }
    // accumulate_low_order_rhs_volume! (:139-173), graph_viscosity (rhs_utils.jl:446-461)
#pragma omp parallel for schedule(static)
    for (int k = 0; k < K; ++k) {
      for (auto [i, j] : Srs0_nnz) {
        const V4& u_i = Uq[i + (size_t)Nq * k];
        const V4& u_j = Uq[j + (size_t)Nq * k];
        const V2x4& fi = flux[i + (size_t)Nh * k];
        const V2x4& fj = flux[j + (size_t)Nh * k];
        V2x4 F;
        for (int c = 0; c < 4; ++c) {
          F.x[c] = 0.5 * (fi.x[c] + fj.x[c]);
          F.y[c] = 0.5 * (fi.y[c] + fj.y[c]);
        }
        auto S = Sx0(i, j, k);
        double nn = norm2(S[0], S[1]);
        double n1 = S[0] / nn, n2 = S[1] / nn;
        double ws = jmax(eq.wavespeed(u_i, n1, n2), eq.wavespeed(u_j, -n1, -n2));
        double lij = nn * ws;
        lambda[i + (size_t)Nq * (j + (size_t)Nq * k)] = lij;
        lambda[j + (size_t)Nq * (i + (size_t)Nq * k)] = lij;
        V4 visc = scal(lij, sub(u_j, u_i));
        V4 zero{0.0, 0.0, 0.0, 0.0};
        V2x4 lD;
        if (std::fabs(S[0]) > 1e-10) {
          lD.x = visc;
          lD.y = zero;
        } else {
          lD.x = zero;
          lD.y = visc;
        }
        V2x4 SF;
        for (int c = 0; c < 4; ++c) {
          SF.x[c] = 2.0 * S[0] * F.x[c] - lD.x[c];
          SF.y[c] = 2.0 * S[1] * F.y[c] - lD.y[c];
        }
        V2x4& Qi = Q0F1[i + (size_t)Nq * k];
        V2x4& Qj = Q0F1[j + (size_t)Nq * k];
        Qi.x = add(Qi.x, SF.x);
        Qi.y = add(Qi.y, SF.y);
        Qj.x = add(Qj.x, neg(SF.x));
        Qj.y = add(Qj.y, neg(SF.y));
      }
      for (int i = 0; i < Nq; ++i) {
        V2x4& r = rhsxyL[i + (size_t)Nq * k];
        r.x = sub(r.x, Q0F1[i + (size_t)Nq * k].x);
        r.y = sub(r.y, Q0F1[i + (size_t)Nq * k].y);
      }
    }
    // accumulate_low_order_rhs_surface! (:175-204), LF placement rhs_utils.jl:415-435
#pragma omp parallel for schedule(static)
    for (int k = 0; k < K; ++k) {
      for (int f = 0; f < Nfp; ++f) {
        size_t fk = f + (size_t)Nfp * k;
        int iP, kP;
        face_of(mapP[fk], iP, kP);
        auto B = Bx(f, k);
        double nn = norm2(B[0], B[1]);
        lambdaB[fk] = 0.5 * nn * jmax(wavespeed_f[fk], wavespeed_f[iP + (size_t)Nfp * kP]);
        V2x4 fP = eq.fluxes(uP_L[fk]);
        const V2x4& fM = flux[Nq + f + (size_t)Nh * k];
        V2x4 fs;
        for (int c = 0; c < 4; ++c) {
          fs.x[c] = 0.5 * (fM.x[c] + fP.x[c]);
          fs.y[c] = 0.5 * (fM.y[c] + fP.y[c]);
        }
        V2x4 BF;
        BF.x = scal(B[0], fs.x);
        BF.y = scal(B[1], fs.y);
        V4 lf = scal(lambdaB[fk], sub(uP_L[fk], Uf[fk]));
        if (f < 2 * N1D) {
          BF.x = sub(BF.x, lf);
          fs.x = sub(fs.x, divs(lf, B[0]));
        } else {
          BF.y = sub(BF.y, lf);
          fs.y = sub(fs.y, divs(lf, B[1]));
        }
        BF_L[fk] = BF;
        fstar_L[fk] = fs;
        V2x4& r = rhsxyL[fq2q[f] + (size_t)Nq * k];
        r.x = sub(r.x, BF.x);
        r.y = sub(r.y, BF.y);
      }
    }
    // scale_low_order_rhs_by_mass! (:206-220)
#pragma omp parallel for schedule(static)
    for (int k = 0; k < K; ++k)
      for (int i = 0; i < Nq; ++i) {
        size_t ik = i + (size_t)Nq * k;
        double wJq = Jq[ik] * wq[i];
        rhsxyL[ik].x = divs(rhsxyL[ik].x, wJq);
        rhsxyL[ik].y = divs(rhsxyL[ik].y, wJq);
        rhsL[ik] = add(rhsxyL[ik].x, rhsxyL[ik].y);
      }
    // calculate_lambda_and_low_order_CFL! (:222-243), lambda_i (:263-281)
    if (nstage == 1) {
      double dt_init = jmin(prm.CFL * prm.dt0, prm.T - t);
      double dtmin = dt_init;
#pragma omp parallel
      {
        double dtl = dt_init;
#pragma omp for schedule(static)
        for (int k = 0; k < K; ++k)
          for (int i = 0; i < Nq; ++i) {
            double li = 0.0;
            for (int j = 0; j < Nq; ++j) li += lambda[i + (size_t)Nq * (j + (size_t)Nq * k)];
            for (int f : q2fq[i]) {
              const size_t fk = f + (size_t)Nfp * k;
              if (lf_proj) {  // lambda_B_CFL(::LaxFriedrichsOnProjectedVal) (:305-309)
                auto B = Bx(f, k);
                const double nn = norm2(B[0], B[1]);
                li += find_alpha(Uq[fq2q[f] + (size_t)Nq * k], u_tilde[Nq + f + (size_t)Nh * k]) * lambdaB[fk] +
                      0.5 * nn * wavespeed_f[fk];
              } else {
                li += lambdaB[fk];
              }
            }
            double wJq = Jq[i + (size_t)Nq * k] * wq[i];
            dtl = jmin(dtl, prm.CFL * 0.5 * wJq / li);
          }
#pragma omp critical
        dtmin = jmin(dtmin, dtl);
      }
      dt = dtmin;
    }
    return dt;
  }

  // find_alpha (low_order_graph_viscosity.jl:316-345): KPP 1; Euler, the alpha with
  // alpha ui - uitilde of positive density and internal energy, doubling then bisecting
  double find_alpha(const V4& ui, const V4& ut) const {
    if (eq.kpp) return 1.0;
    const double POSTOL = prm.POSTOL;
    auto ok = [&](double al) {
      V4 sub_ = sub(scal(al, ui), ut);
      return sub_[0] > POSTOL && eq.rhoe_ufun(sub_) > POSTOL;
    };
    double alphaL = 0.0, alphaR = 1.0;
    while (!ok(alphaR)) alphaR = 2 * alphaR;
    const int maxit = 50;
    double iter = 0.0;
    const double tolerance = 1e-8;
    while (iter < maxit || (alphaL - alphaR) > tolerance) {
      const double alphaM = (alphaL + alphaR) / 2;
      if (ok(alphaM)) alphaR = alphaM;
      else alphaL = alphaM;
      iter = iter + 1;
    }
    return alphaR;
  }

  // ---------------------------------------------------------------------------
  // rhs_fluxdiff! (flux_differencing.jl:4-37)
  // ---------------------------------------------------------------------------
  void rhs_fluxdiff(double t, int nstage) {
    // calculate_primitive_variables! (:39-70; KPP only gathers uP, :72-88)
#pragma omp parallel for schedule(static)
    for (int k = 0; k < K; ++k)
      for (int i = 0; i < Nh && !eq.kpp; ++i) {
        size_t ik = i + (size_t)Nh * k;
        psi_tilde[ik] = eq.psi_ufun(u_tilde[ik]);
        beta[ik] = eq.betafun(u_tilde[ik]);
        rholog[ik] = std::log(u_tilde[ik][0]);
        betalog[ik] = std::log(beta[ik]);
      }
#pragma omp parallel for schedule(static)
    for (int k = 0; k < K; ++k)
      for (int f = 0; f < Nfp; ++f) {
        size_t fk = f + (size_t)Nfp * k;
        int iP, kP;
        face_of(mapP[fk], iP, kP);
        size_t src = Nq + iP + (size_t)Nh * kP;
        uP_H[fk] = u_tilde[src];
        betaP[fk] = beta[src];
        rhologP[fk] = rholog[src];
        betalogP[fk] = betalog[src];
      }
    // calculate_interface_dissipation_coeff! (:90-114)
#pragma omp parallel for schedule(static)
    for (int k = 0; k < K; ++k)
      for (int f = 0; f < Nfp; ++f) {
        size_t fk = f + (size_t)Nfp * k;
        auto B = Bx(f, k);
        double nn = norm2(B[0], B[1]);
        lam[fk] = eq.wavespeed(u_tilde[Nq + f + (size_t)Nh * k], B[0] / nn, B[1] / nn);
        LFc[fk] = 0.5 * nn;
      }
#pragma omp parallel for schedule(static)
    for (int k = 0; k < K; ++k)
      for (int f = 0; f < Nfp; ++f) {
        size_t fk = f + (size_t)Nfp * k;
        LFc[fk] = LFc[fk] * jmax(lam[fk], lam[mapP[fk] - 1]);
      }
    // enforce_BC! (:116-151) plus the wall / moving-shock extension
    for (int64_t m : mapI) LFc[m - 1] = 0.0;
    for (int64_t m : mapO) LFc[m - 1] = 0.0;
    for (int64_t m : mapS) LFc[m - 1] = 0.0;
    auto set_P = [&](size_t io, const V4& u) {
      uP_H[io] = u;
      betaP[io] = eq.betafun(u);
      rhologP[io] = std::log(u[0]);
      betalogP[io] = std::log(betaP[io]);
    };
    for (size_t i = 0; i < mapI.size(); ++i) set_P(mapI[i] - 1, Ival[i]);
    for (size_t i = 0; i < mapO.size(); ++i) {
      int iP, kP;
      face_of(mapO[i], iP, kP);
      set_P(mapO[i] - 1, Uq[fq2q[iP] + (size_t)Nq * kP]);
    }
    for (size_t i = 0; i < mapW.size(); ++i) {
      int64_t lin = mapW[i] - 1;
      auto n = unit_normal(lin);
      int f = (int)(lin % Nfp), k = (int)(lin / Nfp);
      set_P(lin, reflect(u_tilde[Nq + f + (size_t)Nh * k], n[0], n[1]));
    }
    for (size_t i = 0; i < mapS.size(); ++i) set_P(mapS[i] - 1, shock_state((int64_t)i, t));
    // clear_flux_differencing_cache! (:153-162)
    std::fill(QF1.begin(), QF1.end(), V2x4{});
    // flux_differencing_volume! (:164-176), U(::Dim2,...) (:186-191), accumulate_QF1! (:201-211)
#pragma omp parallel for schedule(static)
    for (int k = 0; k < K; ++k) {
      for (auto [i, j] : Srsh_nnz) {
        size_t ik = i + (size_t)Nh * k, jk = j + (size_t)Nh * k;
        const V4& ui = u_tilde[ik];
        const V4& uj = u_tilde[jk];
        auto S = Sx(i, j, k);
        V2x4 F;
        if (eq.kpp) {
          F = Euler::fS_kpp(ui[0], uj[0]);
        } else {
          double Ui[6] = {ui[0], ui[1] / ui[0], ui[2] / ui[0], beta[ik], rholog[ik], betalog[ik]};
          double Uj[6] = {uj[0], uj[1] / uj[0], uj[2] / uj[0], beta[jk], rholog[jk], betalog[jk]};
          F = eq.fS(Ui, Uj);
        }
        V2x4 SF;
        SF.x = scal(S[0], F.x);
        SF.y = scal(S[1], F.y);
        QF1[ik].x = add(QF1[ik].x, SF.x);
        QF1[ik].y = add(QF1[ik].y, SF.y);
        QF1[jk].x = add(QF1[jk].x, neg(SF.x));
        QF1[jk].y = add(QF1[jk].y, neg(SF.y));
      }
    }
    // flux_differencing_surface! (:223-247), LaxFriedrichsOnProjectedVal (:262-272)
#pragma omp parallel for schedule(static)
    for (int k = 0; k < K; ++k)
      for (int f = 0; f < Nfp; ++f) {
        size_t fk = f + (size_t)Nfp * k;
        const V4& uf = u_tilde[Nq + f + (size_t)Nh * k];
        V2x4 ff = eq.fluxes(uf), fP = eq.fluxes(uP_H[fk]);
        V2x4 fs;
        for (int c = 0; c < 4; ++c) {
          fs.x[c] = 0.5 * (ff.x[c] + fP.x[c]);
          fs.y[c] = 0.5 * (ff.y[c] + fP.y[c]);
        }
        auto B = Bx(f, k);
        V2x4 BF;
        BF.x = scal(B[0], fs.x);
        BF.y = scal(B[1], fs.y);
        V4 lf = scal(LFc[fk], sub(uP_H[fk], uf));
        if (f < 2 * N1D) {
          BF.x = sub(BF.x, lf);
          fs.x = sub(fs.x, divs(lf, B[0]));
        } else {
          BF.y = sub(BF.y, lf);
          fs.y = sub(fs.y, divs(lf, B[1]));
        }
        BF_H[fk] = BF;
        fstar_H[fk] = fs;
      }
    // assemble_rhs! (:331-361), project_flux_difference_to_quad_unlimited! (:274-281):
    // generic mat-vec C[i] = sum_j A[i,j]*B[j] accumulated column by column.
    // With any theta < 1 on the element (is_Vf_limited, :316-318), the lift uses
    // (1/wq) [I, Vf_new'] with Vf_new = theta Vf + (1 - theta) Vf_low per face row
    // (project_flux_difference_to_quad!(::ScaledExtrapolation), :288-314)
    const int s = nstage - 1;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < K; ++k) {
      const double* th = &theta_local[(size_t)Nfp * (k + (size_t)K * s)];
      bool limited = false;
      for (int f = 0; f < Nfp; ++f) limited = limited || th[f] < 1.0;
      std::vector<double> Mh;
      if (limited) {
        Mh.assign((size_t)Nq * Nh, 0.0);
        for (int i = 0; i < Nq; ++i) {
          const double rw = 1 / wq[i];
          Mh[i + (size_t)Nq * i] = rw * 1.0;
          for (int f = 0; f < Nfp; ++f)
            Mh[i + (size_t)Nq * (Nq + f)] = rw * (th[f] * Vf[f + (size_t)Nfp * i] + (1 - th[f]) * Vf_low[f + (size_t)Nfp * i]);
        }
      }
      const double* MVh = limited ? Mh.data() : MinvVhT.data();
      const double* MVf = limited ? Mh.data() + (size_t)Nq * Nq : MinvVfT.data();
      for (int i = 0; i < Nq; ++i) {
        V2x4 a{}, b{};
        for (int j = 0; j < Nh; ++j) {
          double m = MVh[i + (size_t)Nq * j];
          const V2x4& q = QF1[j + (size_t)Nh * k];
          a.x = add(a.x, scal(m, q.x));
          a.y = add(a.y, scal(m, q.y));
        }
        for (int f = 0; f < Nfp; ++f) {
          double m = MVf[i + (size_t)Nq * f];
          const V2x4& q = BF_H[f + (size_t)Nfp * k];
          b.x = add(b.x, scal(m, q.x));
          b.y = add(b.y, scal(m, q.y));
        }
        MinvVhTQF1[i + (size_t)Nq * k] = a;
        MinvVfTBF1[i + (size_t)Nq * k] = b;
        size_t ik = i + (size_t)Nq * k;
        double J = Jq[ik];
        rhsxyH[ik].x = divs(neg(add(a.x, b.x)), J);
        rhsxyH[ik].y = divs(neg(add(a.y, b.y)), J);
        rhsH[ik] = add(rhsxyH[ik].x, rhsxyH[ik].y);
      }
    }
  }

  // ---------------------------------------------------------------------------
  // Subcell limiter (limiter.jl:20-56; subcell.jl; limiter_utils.jl)
  // ---------------------------------------------------------------------------
  // limiter_utils.jl:141-146
  static void rhoe_quadratic_coefficients(const V4& U, const V4& P, double Lrhoe, double& a, double& b, double& c) {
    a = P[0] * P[3] - 1.0 / 2.0 * (P[1] * P[1] + P[2] * P[2]);
    b = U[3] * P[0] + U[0] * P[3] - U[1] * P[1] - U[2] * P[2] - P[0] * Lrhoe;
    c = U[3] * U[0] - 1.0 / 2.0 * (U[1] * U[1] + U[2] * U[2]) - U[0] * Lrhoe;
  }
  // limiter_utils.jl:108-132
  double rhoe_quadratic_solve(const V4& UL, const V4& P, double Lrhoe) const {
    if (Lrhoe == kInf) return 1.0;
    double a, b, c;
    rhoe_quadratic_coefficients(UL, P, Lrhoe, a, b, c);
    double l_eps_ij = 1.0;
    if (b * b - 4.0 * a * c >= 0.0) {
      double r1 = (-b + std::sqrt(b * b - 4.0 * a * c)) / (2.0 * a);
      double r2 = (-b - std::sqrt(b * b - 4.0 * a * c)) / (2.0 * a);
      double Z = prm.ZEROTOL;
      if (r1 > Z && r2 > Z) {
        l_eps_ij = jmin(r1, r2);
      } else if (r1 > Z && r2 < -Z) {
        l_eps_ij = r1;
      } else if (r2 > Z && r1 < -Z) {
        l_eps_ij = r2;
      }
    }
    return l_eps_ij;
  }
  // limiter_utils.jl:82-96
  double limiting_param_bound_rho_rhoe(const V4& U, const V4& P, double Lrho, double Lrhoe, double Urho, double Urhoe) const {
    double l = 1.0;
    if (U[0] + P[0] < Lrho) l = jmax((Lrho - U[0]) / P[0], 0.0);
    if (U[0] + P[0] > Urho) l = jmin(l, jmax((Urho - U[0]) / P[0], 0.0));
    l = jmin(jmin(l, rhoe_quadratic_solve(U, P, Lrhoe)), rhoe_quadratic_solve(U, P, Urhoe));
    return l;
  }
  // limiter_utils.jl:66-70 with the 5-tuple bound (Lrho, Lrhoe, Lphi, Urho, Urhoe)
  // of subcell.jl:299,311,327,339. The reference destructures it into four names.
  double limiting_param(const V4& UL, const V4& P, const double bv[5]) const {
    if (prm.reference_semantics)
      return limiting_param_bound_rho_rhoe(UL, P, bv[0], bv[1], bv[2], bv[3]);
    return limiting_param_bound_rho_rhoe(UL, P, bv[0], bv[1], bv[3], bv[4]);
  }

  bool gauss() const { return prm.approximation_basis == P2DE_BASIS_GAUSS; }
  bool scaled_extrapolation() const {
    return prm.entropyproj_limiter == P2DE_ENTROPYPROJ_NODEWISE_SCALED_EXTRAPOLATION;
  }

  // bound families (Solver.jl:47-62)
  bool bound_is(std::initializer_list<int> l) const {
    for (int b : l)
      if (prm.bound_type == b) return true;
    return false;
  }
  bool tvd() const {
    return bound_is({P2DE_BOUND_TVD, P2DE_BOUND_TVD_AND_CELL_ENTROPY, P2DE_BOUND_TVD_AND_MIN_ENTROPY,
                     P2DE_BOUND_TVD_AND_RELAXED_MIN_ENTROPY, P2DE_BOUND_TVD_AND_RELAXED_CELL_ENTROPY});
  }
  bool cell_entropy() const {
    return bound_is({P2DE_BOUND_POSITIVITY_AND_CELL_ENTROPY, P2DE_BOUND_TVD_AND_CELL_ENTROPY,
                     P2DE_BOUND_POSITIVITY_AND_RELAXED_CELL_ENTROPY, P2DE_BOUND_TVD_AND_RELAXED_CELL_ENTROPY});
  }
  bool min_entropy() const {
    return bound_is({P2DE_BOUND_POSITIVITY_AND_MIN_ENTROPY, P2DE_BOUND_POSITIVITY_AND_RELAXED_MIN_ENTROPY,
                     P2DE_BOUND_TVD_AND_MIN_ENTROPY, P2DE_BOUND_TVD_AND_RELAXED_MIN_ENTROPY});
  }
  bool relaxed() const {
    return bound_is({P2DE_BOUND_POSITIVITY_AND_RELAXED_MIN_ENTROPY, P2DE_BOUND_TVD_AND_RELAXED_MIN_ENTROPY,
                     P2DE_BOUND_POSITIVITY_AND_RELAXED_CELL_ENTROPY, P2DE_BOUND_TVD_AND_RELAXED_CELL_ENTROPY});
  }

  // s_modified_ufun (compressible_Navier_Stokes.jl:80-85): rhoe rho^(-gamma)
  double s_modified(const V4& U) const { return eq.rhoe_ufun(U) * std::pow(U[0], -eq.gamma); }

  // limiting_param(::SubcellLimiter, min-entropy bounds) (limiter_utils.jl:19-24): the
  // 5-tuple read as 5 names; the positivity factor, then bisection (nonlinear_solvers.jl:3-20)
  // for phi(UL + l P) >= Lphi - POSTOL over [0, lpos] (limiting_param_bound_phi, :43-50)
  double limiting_param_min_entropy(const V4& UL, const V4& P, const double bv[5]) const {
    const double lpos = limiting_param_bound_rho_rhoe(UL, P, bv[0], bv[1], bv[3], bv[4]);
    const double Lphi = bv[2];
    auto f = [&](double l) { return s_modified(add(UL, scal(l, P))) >= Lphi - prm.POSTOL; };
    double x_valid = 0.0, x_invalid = lpos;
    if (f(x_invalid)) return x_invalid;
    for (int iter = 0; iter <= 20; ++iter) {
      const double x_new = 0.5 * (x_valid + x_invalid);
      if (f(x_new)) x_valid = x_new;
      else x_invalid = x_new;
    }
    return x_valid;
  }

  // low_order_stencil (limiter_utils.jl:222-231): the r-neighbours, then the s-neighbours,
  // across an element face through quad_index_to_quad_index_P
  void low_order_stencil(int q, int k, int kk[4], int qq[4]) const {
    const int i = q % N1D, j = q / N1D;
    if (i - 1 >= 0) { qq[0] = q - 1; kk[0] = k; } else qq[0] = quad_index_to_quad_index_P(q, k, 1, kk[0]);
    if (i + 1 <= N) { qq[1] = q + 1; kk[1] = k; } else qq[1] = quad_index_to_quad_index_P(q, k, 1, kk[1]);
    if (j - 1 >= 0) { qq[2] = q - N1D; kk[2] = k; } else qq[2] = quad_index_to_quad_index_P(q, k, 2, kk[2]);
    if (j + 1 <= N) { qq[3] = q + N1D; kk[3] = k; } else qq[3] = quad_index_to_quad_index_P(q, k, 2, kk[3]);
  }

  // low_order_stencil(::Dim1) (limiter_utils.jl:214-220): left, right neighbour; across an
  // element face through quad_index_to_quad_index_P(::Dim1) (:184-195)
  void low_order_stencil_1d(int q, int k, int kk[2], int qq[2]) const {
    auto across = [&](int& kP) {
      int iP;
      face_of(mapP[q2fq[q][0] + (size_t)Nfp * k], iP, kP);
      return fq2q[iP];
    };
    if (q - 1 >= 0) { qq[0] = q - 1; kk[0] = k; } else qq[0] = across(kk[0]);
    if (q + 1 <= N) { qq[1] = q + 1; kk[1] = k; } else qq[1] = across(kk[1]);
  }
  int stencil(int q, int k, int kk[4], int qq[4]) const {
    if (dim1) {
      low_order_stencil_1d(q, k, kk, qq);
      return 2;
    }
    low_order_stencil(q, k, kk, qq);
    return 4;
  }

  // initialize_s_modified! (subcell.jl:21-35) and initialize_lower_bound!(::Dim2) (:53-72):
  // Lphi = eps_k min(phi over the node and its stencil) + (1 - eps_k) min phi(initial)
  std::vector<double> s_mod, lbound_s_modified;
  double s_modified_min = 0.0;  // zeros(Float64, 1) until t == t0 at stage 1
  void initialize_entropy_bounds(double t, int nstage) {
    s_mod.assign((size_t)Nq * K, 0.0);
    lbound_s_modified.assign((size_t)Nq * K, 0.0);
#pragma omp parallel for schedule(static)
    for (size_t i = 0; i < s_mod.size(); ++i) s_mod[i] = s_modified(Uq[i]);
    if (t == prm.t0 && nstage == 1) {
      double m = s_mod[0];
      for (size_t i = 1; i < s_mod.size(); ++i) m = jmin(m, s_mod[i]);
      s_modified_min = m;
    }
#pragma omp parallel for schedule(static)
    for (int k = 0; k < K; ++k) {
      const double epsk = smooth_factor[k];
      for (int q = 0; q < Nq; ++q) {
        int kk[4], qq[4];
        const int ns = stencil(q, k, kk, qq);
        double lb = s_mod[q + (size_t)Nq * k];
        for (int t4 = 0; t4 < ns; ++t4) lb = jmin(lb, s_mod[qq[t4] + (size_t)Nq * kk[t4]]);
        lbound_s_modified[q + (size_t)Nq * k] = epsk * lb + (1 - epsk) * s_modified_min;
      }
    }
  }

  // quad_index_to_quad_index_P(::Dim2) (limiter_utils.jl:199-212): the volume node across
  // the face of boundary node q in `direction` (1: r, 2: s); q2fq lists the r-face first
  int quad_index_to_quad_index_P(int q, int k, int direction, int& kP) const {
    const int ir = q % N1D, is = q / N1D;
    int faces[4] = {0, 0, 0, 0}, nf = 0;
    if (ir == 0) faces[nf++] = is;
    if (ir == N) faces[nf++] = N1D + is;
    if (is == 0) faces[nf++] = 2 * N1D + ir;
    if (is == N) faces[nf++] = 3 * N1D + ir;
    const int iface = nf == 1 ? faces[0] : faces[direction - 1];
    int iP;
    face_of(mapP[iface + (size_t)Nfp * k], iP, kP);
    return fq2q[iP];
  }

  // initialize_TVD_bounds!(::Dim2) (subcell.jl:112-141) with low_order_stencil
  // (limiter_utils.jl:222-231); ::Dim1 (:86-110) with the two-point stencil
  std::vector<double> rhoL_tvd, lbound_rho, ubound_rho;
  void initialize_TVD_bounds(double dt) {
    rhoL_tvd.assign((size_t)Nq * K, 0.0);
    lbound_rho.assign((size_t)Nq * K, 0.0);
    ubound_rho.assign((size_t)Nq * K, 0.0);
#pragma omp parallel for schedule(static)
    for (int k = 0; k < K; ++k)
      for (int i = 0; i < Nq; ++i) {
        size_t ik = i + (size_t)Nq * k;
        rhoL_tvd[ik] = Uq[ik][0] + dt * rhsL[ik][0];
      }
#pragma omp parallel for schedule(static)
    for (int k = 0; k < K; ++k)
      for (int q = 0; q < Nq; ++q) {
        int kk[4], qq[4];
        const int ns = stencil(q, k, kk, qq);
        double lb = rhoL_tvd[q + (size_t)Nq * k], ub = lb;
        for (int s = 0; s < ns; ++s) {
          double v = rhoL_tvd[qq[s] + (size_t)Nq * kk[s]];
          lb = jmin(lb, v);
          ub = jmax(ub, v);
        }
        lbound_rho[q + (size_t)Nq * k] = lb;
        ubound_rho[q + (size_t)Nq * k] = ub;
      }
  }

  // apply_rhs_limiter!(::SubcellLimiter) (limiter.jl:20-56)
  void apply_rhs_limiter(double t, double dt, int nstage) {
    const int s = nstage - 1;
    const int N1Dp1 = N1D + 1;
    // smoothness indicator, blending factor (NoShockCapture: 1.0), smoothness factor;
    // initialize_entropy_bounds!: lbound_s_modified = 0.0 except for the min-entropy
    // bounds (subcell.jl:4-19)
    update_smoothness();
    if (eq.kpp) {  // subcell_bound_limiter!(dim, ::KPP) (subcell.jl:389-402): 1 capped by blending
      const int s2 = nstage - 1;
      for (int k = 0; k < K; ++k)
        for (int i = 0; i < Nq + N1D; ++i)
          for (int d = 0; d < 2; ++d) L_local[LL(i, d, k, s2)] = jmin(1.0, blending_factor[k]);
    }
    if (!eq.kpp && min_entropy()) initialize_entropy_bounds(t, nstage);
    if (!eq.kpp && tvd()) initialize_TVD_bounds(dt);
    if (dim1) {
      subcell_limiter_1d(dt, s);
      return;
    }
    // accumulate_f_bar!(::Dim2) (subcell.jl:163-206)
#pragma omp parallel for schedule(static)
    for (int k = 0; k < K; ++k) {
      V4* fxH = &f_bar_H[0][(size_t)(Nq + N1D) * k];
      V4* fxL = &f_bar_L[0][(size_t)(Nq + N1D) * k];
      V4* fyH = &f_bar_H[1][(size_t)(Nq + N1D) * k];
      V4* fyL = &f_bar_L[1][(size_t)(Nq + N1D) * k];
      for (int sj = 0; sj < N1D; ++sj) {
        int iface = sj;
        fxH[0 + N1Dp1 * sj] = BF_H[iface + (size_t)Nfp * k].x;
        fxL[0 + N1Dp1 * sj] = BF_L[iface + (size_t)Nfp * k].x;
        for (int si = 1; si < N1Dp1; ++si) {
          int q = (si - 1) + N1D * sj;
          size_t qk = q + (size_t)Nq * k;
          double wJ = wq[q] * Jq[qk];
          fxH[si + N1Dp1 * sj] = add(fxH[(si - 1) + N1Dp1 * sj], scal(wJ, rhsxyH[qk].x));
          fxL[si + N1Dp1 * sj] = add(fxL[(si - 1) + N1Dp1 * sj], scal(wJ, rhsxyL[qk].x));
        }
      }
      for (int si = 0; si < N1D; ++si) {
        int iface = si + 2 * N1D;
        fyH[si + N1D * 0] = BF_H[iface + (size_t)Nfp * k].y;
        fyL[si + N1D * 0] = BF_L[iface + (size_t)Nfp * k].y;
        for (int sj = 1; sj < N1Dp1; ++sj) {
          int q = si + N1D * (sj - 1);
          size_t qk = q + (size_t)Nq * k;
          double wJ = wq[q] * Jq[qk];
          fyH[si + N1D * sj] = add(fyH[si + N1D * (sj - 1)], scal(wJ, rhsxyH[qk].y));
          fyL[si + N1D * sj] = add(fyL[si + N1D * (sj - 1)], scal(wJ, rhsxyL[qk].y));
        }
      }
    }
    // subcell_bound_limiter!(::Dim2) (subcell.jl:248-349), rho_bound (:378-387)
    const double zeta = prm.zeta;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < K; ++k) {
      if (eq.kpp) continue;  // set above
      std::vector<V4> uL(Nq);
      for (int i = 0; i < Nq; ++i) {
        size_t ik = i + (size_t)Nq * k;
        uL[i] = add(Uq[ik], scal(dt, rhsL[ik]));
      }
      for (int i = 0; i < Nq + N1D; ++i)
        for (int d = 0; d < 2; ++d) L_local[LL(i, d, k, s)] = 1.0;
      const double Urhoe = kInf;
      const V4* fxH = &f_bar_H[0][(size_t)(Nq + N1D) * k];
      const V4* fxL = &f_bar_L[0][(size_t)(Nq + N1D) * k];
      const V4* fyH = &f_bar_H[1][(size_t)(Nq + N1D) * k];
      const V4* fyL = &f_bar_L[1][(size_t)(Nq + N1D) * k];
      auto eval = [&](int q, const V4& dF, double sgn) {
        double wJ = wq[q] * Jq[q + (size_t)Nq * k];
        const V4& u = uL[q];
        // rho_bound (subcell.jl:352-387): TVD or positivity
        double Lrho = zeta * u[0], Urho = kInf;
        if (tvd()) {
          Lrho = lbound_rho[q + (size_t)Nq * k];
          Urho = ubound_rho[q + (size_t)Nq * k];
        }
        const double Lphi = min_entropy() ? lbound_s_modified[q + (size_t)Nq * k] : 0.0;
        double bv[5] = {Lrho, zeta * eq.rhoe_ufun(u), Lphi, Urho, Urhoe};
        V4 P;
        for (int c = 0; c < 4; ++c) P[c] = sgn * 4.0 * dt * dF[c] / wJ;
        return min_entropy() ? limiting_param_min_entropy(u, P, bv) : limiting_param(u, P, bv);
      };
      for (int sj = 0; sj < N1D; ++sj) {
        for (int si = 0; si < N1D; ++si) {
          int q = si + N1D * sj;
          size_t id = LL(si + N1Dp1 * sj, 0, k, s);
          L_local[id] = jmin(L_local[id], eval(q, sub(fxH[si + N1Dp1 * sj], fxL[si + N1Dp1 * sj]), -1.0));
        }
        for (int si = 1; si < N1Dp1; ++si) {
          int q = (si - 1) + N1D * sj;
          size_t id = LL(si + N1Dp1 * sj, 0, k, s);
          L_local[id] = jmin(L_local[id], eval(q, sub(fxH[si + N1Dp1 * sj], fxL[si + N1Dp1 * sj]), 1.0));
        }
      }
      for (int si = 0; si < N1D; ++si) {
        for (int sj = 0; sj < N1D; ++sj) {
          int q = si + N1D * sj;
          size_t id = LL(si + N1D * sj, 1, k, s);
          L_local[id] = jmin(L_local[id], eval(q, sub(fyH[si + N1D * sj], fyL[si + N1D * sj]), -1.0));
        }
        for (int sj = 1; sj < N1Dp1; ++sj) {
          int q = si + N1D * (sj - 1);
          size_t id = LL(si + N1D * sj, 1, k, s);
          L_local[id] = jmin(L_local[id], eval(q, sub(fyH[si + N1D * sj], fyL[si + N1D * sj]), 1.0));
        }
      }
      for (int i = 0; i < Nq + N1D; ++i)
        for (int d = 0; d < 2; ++d) L_local[LL(i, d, k, s)] = jmin(L_local[LL(i, d, k, s)], blending_factor[k]);
    }
    // enforce_ES_subcell! (subcell.jl:462-466) for PositivityAndCellEntropyBound
    if (cell_entropy()) {
      initialize_ES_subcell_limiting();
      enforce_ES_subcell_volume(s);
      if (gauss()) enforce_ES_subcell_interface(s);
      // enforce_ES_subcell_interface!(::LobattoCollocation) is a no-op (subcell.jl:755-757)
    }
    // symmetrize_limiting_parameters!(::Dim2) (subcell.jl:418-456), subcell_index_P_x/y
    // (limiter_utils.jl:179-237). Each element takes the min with its partner across the
    // face; both sides end with the same min whatever the visiting order.
    {
      std::vector<double> Lold(L_local.begin() + (size_t)(Nq + N1D) * 2 * K * s,
                               L_local.begin() + (size_t)(Nq + N1D) * 2 * K * (s + 1));
      auto Lo = [&](int i, int d, int k) { return Lold[(size_t)i + (size_t)(Nq + N1D) * (d + 2 * (size_t)k)]; };
#pragma omp parallel for schedule(static)
      for (int k = 0; k < K; ++k) {
        for (int sj = 0; sj < N1D; ++sj)
          for (int si : {0, N1D}) {
            int iface = (si == 0) ? sj : sj + N1D;
            int iP, kP;
            face_of(mapP[iface + (size_t)Nfp * k], iP, kP);
            int sjP = iP % N1D;
            int siP = (iP / N1D == 0) ? 0 : N1D;
            int idx = si + N1Dp1 * sj, idxP = siP + N1Dp1 * sjP;
            L_local[LL(idx, 0, k, s)] = jmin(Lo(idx, 0, k), Lo(idxP, 0, kP));
          }
        for (int si = 0; si < N1D; ++si)
          for (int sj : {0, N1D}) {
            int iface = (sj == 0) ? si + 2 * N1D : si + 3 * N1D;
            int iP, kP;
            face_of(mapP[iface + (size_t)Nfp * k], iP, kP);
            int siP = iP % N1D;
            int sjP = (iP / N1D == 2) ? 0 : N1D;
            int idx = si + N1D * sj, idxP = siP + N1D * sjP;
            L_local[LL(idx, 1, k, s)] = jmin(Lo(idx, 1, k), Lo(idxP, 1, kP));
          }
      }
    }
    // accumulate_f_bar_limited!(::Dim2) (subcell.jl:841-876), apply_subcell_limiter!(::Dim2) (:894-924)
#pragma omp parallel for schedule(static)
    for (int k = 0; k < K; ++k) {
      size_t o = (size_t)(Nq + N1D) * k;
      for (int j = 0; j < N1D; ++j)
        for (int i = 0; i < N1Dp1; ++i) {
          double l = L_local[LL(i + N1Dp1 * j, 0, k, s)];
          size_t id = o + i + N1Dp1 * j;
          f_bar_lim[0][id] = add(scal(l, f_bar_H[0][id]), scal(1.0 - l, f_bar_L[0][id]));
        }
      for (int i = 0; i < N1D; ++i)
        for (int j = 0; j < N1Dp1; ++j) {
          double l = L_local[LL(i + N1D * j, 1, k, s)];
          size_t id = o + i + N1D * j;
          f_bar_lim[1][id] = add(scal(l, f_bar_H[1][id]), scal(1.0 - l, f_bar_L[1][id]));
        }
      for (int j = 0; j < N1D; ++j)
        for (int i = 0; i < N1D; ++i) {
          int q = i + N1D * j;
          size_t qk = q + (size_t)Nq * k;
          double wJ = wq[q] * Jq[qk];
          V2x4 r;
          r.x = divs(sub(f_bar_lim[0][o + (i + 1) + N1Dp1 * j], f_bar_lim[0][o + i + N1Dp1 * j]), wJ);
          r.y = divs(sub(f_bar_lim[1][o + i + N1D * (j + 1)], f_bar_lim[1][o + i + N1D * j]), wJ);
          rhsxyU[qk] = r;
          rhsU[qk] = add(r.x, r.y);
        }
    }
  }

  // The subcell limiter's Dim1 methods: accumulate_f_bar! (subcell.jl:144-160),
  // subcell_bound_limiter! (:208-246) with rho_bound(dim, ...) where the reference writes
  // rho_bound(dim(solver), bound(solver), ...) (:225, :233; dim is the Dim1 argument there),
  // enforce_ES_subcell! (:462-466) through the Dim1 methods of :468-505 and :567-628 with N
  // entries of dvdf per element, symmetrize_limiting_parameters! (:405-415) across mapP
  // between subcell faces 1 and Nq+1 of the two elements, accumulate_f_bar_limited!
  // (:826-839) and apply_subcell_limiter! (:878-892)
  void subcell_limiter_1d(double dt, int s) {
    const int NS = Nq + N1D;  // rows of L_local
#pragma omp parallel for schedule(static)
    for (int k = 0; k < K; ++k) {
      V4* fH = &f_bar_H[0][(size_t)NS * k];
      V4* fL = &f_bar_L[0][(size_t)NS * k];
      fH[0] = BF_H[0 + (size_t)Nfp * k].x;
      fL[0] = BF_L[0 + (size_t)Nfp * k].x;
      for (int i = 1; i <= Nq; ++i) {
        const size_t qk = (i - 1) + (size_t)Nq * k;
        const double wJ = Jq[qk] * wq[i - 1];
        fH[i] = add(fH[i - 1], scal(wJ, rhsH[qk]));
        fL[i] = add(fL[i - 1], scal(wJ, rhsL[qk]));
      }
    }
    const double zeta = prm.zeta;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < K; ++k) {
      std::vector<V4> uL(Nq);
      for (int i = 0; i < Nq; ++i) {
        const size_t ik = i + (size_t)Nq * k;
        uL[i] = add(Uq[ik], scal(dt, rhsL[ik]));
      }
      for (int i = 0; i < NS; ++i) L_local[LL(i, 0, k, s)] = 1.0;
      const V4* fH = &f_bar_H[0][(size_t)NS * k];
      const V4* fL = &f_bar_L[0][(size_t)NS * k];
      auto eval = [&](int q, const V4& dF, double sgn) {
        const double wJ = wq[q] * Jq[q + (size_t)Nq * k];
        const V4& u = uL[q];
        double Lrho = zeta * u[0], Urho = kInf;
        if (tvd()) {
          Lrho = lbound_rho[q + (size_t)Nq * k];
          Urho = ubound_rho[q + (size_t)Nq * k];
        }
        const double Lphi = min_entropy() ? lbound_s_modified[q + (size_t)Nq * k] : 0.0;
        double bv[5] = {Lrho, zeta * eq.rhoe_ufun(u), Lphi, Urho, kInf};
        V4 P;
        for (int c = 0; c < 4; ++c) P[c] = sgn * 2.0 * dt * dF[c] / wJ;
        return min_entropy() ? limiting_param_min_entropy(u, P, bv) : limiting_param(u, P, bv);
      };
      for (int i = 0; i < Nq; ++i) {
        double& l = L_local[LL(i, 0, k, s)];
        l = jmin(l, eval(i, sub(fH[i], fL[i]), -1.0));
      }
      for (int i = 1; i <= Nq; ++i) {
        double& l = L_local[LL(i, 0, k, s)];
        l = jmin(l, eval(i - 1, sub(fH[i], fL[i]), 1.0));
      }
      for (int i = 0; i < NS; ++i) L_local[LL(i, 0, k, s)] = jmin(L_local[LL(i, 0, k, s)], blending_factor[k]);
    }
    if (cell_entropy()) {
      initialize_ES_subcell_limiting_1d();
      enforce_ES_subcell_volume_1d(s);
    }
    {
      std::vector<double> Lold(L_local.begin() + (size_t)NS * K * s, L_local.begin() + (size_t)NS * K * (s + 1));
#pragma omp parallel for schedule(static)
      for (int k = 0; k < K; ++k)
        for (int f = 0; f < Nfp; ++f) {
          int iP, kP;
          face_of(mapP[f + (size_t)Nfp * k], iP, kP);
          const int si = f == 0 ? 0 : Nq, siP = iP == 0 ? 0 : Nq;
          L_local[LL(si, 0, k, s)] = jmin(Lold[si + (size_t)NS * k], Lold[siP + (size_t)NS * kP]);
        }
    }
#pragma omp parallel for schedule(static)
    for (int k = 0; k < K; ++k) {
      const size_t o = (size_t)NS * k;
      for (int i = 0; i <= Nq; ++i) {
        const double l = L_local[LL(i, 0, k, s)];
        f_bar_lim[0][o + i] = add(scal(l, f_bar_H[0][o + i]), scal(1.0 - l, f_bar_L[0][o + i]));
      }
      for (int i = 0; i < Nq; ++i) {
        const size_t ik = i + (size_t)Nq * k;
        const double wJ = wq[i] * Jq[ik];
        rhsU[ik] = divs(sub(f_bar_lim[0][o + i + 1], f_bar_lim[0][o + i]), wJ);
      }
    }
  }

  // initialize_ES_subcell_limiting!(::Dim1) (subcell.jl:468-505)
  void initialize_ES_subcell_limiting_1d() {
    const int NS = Nq + N1D;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < K; ++k) {
      for (int i = 0; i < Nq; ++i) vq[i + (size_t)Nq * k] = eq.v_ufun(Uq[i + (size_t)Nq * k]);
      double sB = 0.0;
      for (int f = 0; f < Nfp; ++f) {
        const size_t fk = f + (size_t)Nfp * k;
        const V4& uf = Uq[fq2q[f] + (size_t)Nq * k];
        vf[fk] = eq.v_ufun(uf);
        psif[fk] = eq.psi_ufun(uf);
        sB = sB + Bx(f, k)[0] * psif[fk][0];
      }
      sum_Bpsi[k] = {sB, 0.0};
      const V4* v = &vq[(size_t)Nq * k];
      const V4* fH = &f_bar_H[0][(size_t)NS * k];
      const V4* fL = &f_bar_L[0][(size_t)NS * k];
      double* d = &dvdf[0][(size_t)N * k];
      double sx = 0.0;
      for (int si = 1; si <= N; ++si) {
        const V4 df = sub(fH[si], fL[si]);
        const V4 dv = sub(v[si - 1], v[si]);
        d[si - 1] = vsum(vmul(dv, df));
        sx += vsum(vmul(dv, fL[si]));
      }
      sum_dvfbarL[k] = {sx, 0.0};
    }
  }

  // enforce_ES_subcell_volume!(::Dim1) (subcell.jl:567-628), rhs_es (:746-753)
  void enforce_ES_subcell_volume_1d(int s) {
    const int M = N;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < K; ++k) {
      const double* d = &dvdf[0][(size_t)M * k];
      auto L = [&](int si) -> double& { return L_local[LL(si, 0, k, s)]; };
      double sum = 0.0;
      for (int si = 1; si <= N; ++si) sum += L(si) * d[si - 1];
      double rhs = sum_Bpsi[k][0] - sum_dvfbarL[k][0];
      if (relaxed()) rhs = (1 - prm.bound_beta * smooth_factor[k]) * rhs;
      const double est = sum - rhs;
      const double tol = jmax(0.0, sum_dvfbarL[k][0] - sum_Bpsi[k][0]);
      if (!(est > tol)) continue;
      std::vector<std::pair<double, int>> order(M);
      for (int i = 0; i < M; ++i) order[i] = {d[i], i + 1};
      std::sort(order.begin(), order.end(), [](const std::pair<double, int>& a, const std::pair<double, int>& b) {
        if (jisless(b.first, a.first)) return true;
        if (jisless(a.first, b.first)) return false;
        return b.second < a.second;
      });
      int curr = 1;
      double lhs = sum;
      while (lhs > rhs + tol && curr <= Nq - 1) {
        const int idx = order[curr - 1].second;  // subcell face idx + 1 (1-based)
        if (d[idx - 1] < prm.ZEROTOL) break;
        lhs = lhs - L(idx) * d[idx - 1];
        curr += 1;
      }
      for (int i = 1; i <= curr - 1; ++i) {
        const int idx = order[i - 1].second;
        const double l_new = (i == curr - 1) ? jmax((rhs + tol - lhs) / d[idx - 1], 0.0) : 0.0;
        L(idx) = jmin(L(idx), l_new);
      }
    }
  }

  // initialize_ES_subcell_limiting!(::Dim2) (subcell.jl:508-564)
  void initialize_ES_subcell_limiting() {
    const int N1Dm1 = N1D - 1, N1Dp1 = N1D + 1;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < K; ++k) {
      for (int i = 0; i < Nq; ++i) vq[i + (size_t)Nq * k] = eq.v_ufun(Uq[i + (size_t)Nq * k]);
      std::array<double, 2> sB{0.0, 0.0};
      for (int f = 0; f < Nfp; ++f) {
        size_t fk = f + (size_t)Nfp * k;
        const V4& uf = Uq[fq2q[f] + (size_t)Nq * k];
        vf[fk] = eq.v_ufun(uf);
        psif[fk] = eq.psi_ufun(uf);
        auto B = Bx(f, k);
        sB[0] = sB[0] + B[0] * psif[fk][0];
        sB[1] = sB[1] + B[1] * psif[fk][1];
      }
      sum_Bpsi[k] = sB;
      const V4* v = &vq[(size_t)Nq * k];
      const V4* fxH = &f_bar_H[0][(size_t)(Nq + N1D) * k];
      const V4* fxL = &f_bar_L[0][(size_t)(Nq + N1D) * k];
      const V4* fyH = &f_bar_H[1][(size_t)(Nq + N1D) * k];
      const V4* fyL = &f_bar_L[1][(size_t)(Nq + N1D) * k];
      double* dx = &dvdf[0][(size_t)(Nq - N1D) * k];
      double* dy = &dvdf[1][(size_t)(Nq - N1D) * k];
      double sx = 0.0;
      for (int sj = 0; sj < N1D; ++sj)
        for (int si = 1; si < N1D; ++si) {
          const V4& fL = fxL[si + N1Dp1 * sj];
          V4 df = sub(fxH[si + N1Dp1 * sj], fL);
          V4 dv = sub(v[(si - 1) + N1D * sj], v[si + N1D * sj]);
          dx[(si - 1) + N1Dm1 * sj] = vsum(vmul(dv, df));
          sx += vsum(vmul(dv, fL));
        }
      double sy = 0.0;
      for (int si = 0; si < N1D; ++si)
        for (int sj = 1; sj < N1D; ++sj) {
          const V4& fL = fyL[si + N1D * sj];
          V4 df = sub(fyH[si + N1D * sj], fL);
          V4 dv = sub(v[si + N1D * (sj - 1)], v[si + N1D * sj]);
          dy[si + N1D * (sj - 1)] = vsum(vmul(dv, df));
          sy += vsum(vmul(dv, fL));
        }
      sum_dvfbarL[k] = {sx, sy};
    }
  }

  // enforce_ES_subcell_interface!(::Dim2, ::GaussCollocation) (subcell.jl:759-823) with
  // solve_l_es_interface! (:811-817): per boundary subcell face, the largest l on the
  // bisection grid of [0, min(L, L_partner)] with l dvfH + (1 - l) dvfL <= dpsi, written to
  // the element's own factor. The reference runs this under @batch, where an element reads
  // its partner's factor before or after the partner's own update; here elements go in
  // ascending order, as on one thread.
  void enforce_ES_subcell_interface(int s) {
    const int N1Dp1 = N1D + 1;
    auto solve = [&](double& Lown, double Lpar, double dvfH, double dvfL, double dpsi) {
      const double l = jmin(Lown, Lpar);
      auto f = [&](double li) { return li * dvfH + (1 - li) * dvfL <= dpsi; };
      double x_valid = 0.0, x_invalid = l;
      if (f(x_invalid)) {
        Lown = x_invalid;
        return;
      }
      for (int iter = 0; iter <= 20; ++iter) {
        const double x_new = 0.5 * (x_valid + x_invalid);
        if (f(x_new)) x_valid = x_new;
        else x_invalid = x_new;
      }
      Lown = x_valid;
    };
    for (int k = 0; k < K; ++k) {
      for (int sj = 0; sj < N1D; ++sj)
        for (int si : {0, N1D}) {
          const int iface = (si == 0) ? sj : sj + N1D;
          const size_t fk = iface + (size_t)Nfp * k, fP = (size_t)(mapP[fk] - 1);
          int iP, kP;
          face_of(mapP[fk], iP, kP);
          const int sjP = iP % N1D, siP = (iP / N1D == 0) ? 0 : N1D;
          const V4 dv = sub(vf[fk], vf[fP]);
          const double dpsi = psif[fk][0] - psif[fP][0];
          solve(L_local[LL(si + N1Dp1 * sj, 0, k, s)], L_local[LL(siP + N1Dp1 * sjP, 0, kP, s)],
                vsum(vmul(dv, fstar_H[fk].x)), vsum(vmul(dv, fstar_L[fk].x)), dpsi);
        }
      for (int si = 0; si < N1D; ++si)
        for (int sj : {0, N1D}) {
          const int iface = (sj == 0) ? si + 2 * N1D : si + 3 * N1D;
          const size_t fk = iface + (size_t)Nfp * k, fP = (size_t)(mapP[fk] - 1);
          int iP, kP;
          face_of(mapP[fk], iP, kP);
          const int siP = iP % N1D, sjP = (iP / N1D == 2) ? 0 : N1D;
          const V4 dv = sub(vf[fk], vf[fP]);
          const double dpsi = psif[fk][1] - psif[fP][1];
          solve(L_local[LL(si + N1D * sj, 1, k, s)], L_local[LL(siP + N1D * sjP, 1, kP, s)],
                vsum(vmul(dv, fstar_H[fk].y)), vsum(vmul(dv, fstar_L[fk].y)), dpsi);
        }
    }
  }

  // enforce_ES_subcell_volume!(::Dim2) (subcell.jl:630-744), rhs_es (:746-748)
  void enforce_ES_subcell_volume(int s) {
    const int N1Dm1 = N1D - 1, N1Dp1 = N1D + 1;
    const int M = Nq - N1D;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < K; ++k) {
      const double* dx = &dvdf[0][(size_t)M * k];
      const double* dy = &dvdf[1][(size_t)M * k];
      auto Lx = [&](int si, int sj) -> double& { return L_local[LL(si + N1Dp1 * sj, 0, k, s)]; };
      auto Ly = [&](int si, int sj) -> double& { return L_local[LL(si + N1D * sj, 1, k, s)]; };
      double sumx = 0.0;
      for (int sj = 0; sj < N1D; ++sj)
        for (int si = 1; si < N1D; ++si) sumx += Lx(si, sj) * dx[(si - 1) + N1Dm1 * sj];
      // rhs_es: relaxed bounds scale the target by 1 - beta eps_k (subcell.jl:750-753)
      const double scale = relaxed() ? 1 - prm.bound_beta * smooth_factor[k] : 1.0;
      double rhsx = sum_Bpsi[k][0] - sum_dvfbarL[k][0];
      if (relaxed()) rhsx = scale * rhsx;
      double est_x = sumx - rhsx;
      double sumy = 0.0;
      for (int si = 0; si < N1D; ++si)
        for (int sj = 1; sj < N1D; ++sj) sumy += Ly(si, sj) * dy[si + N1D * (sj - 1)];
      double rhsy = sum_Bpsi[k][1] - sum_dvfbarL[k][1];
      if (relaxed()) rhsy = scale * rhsy;
      double est_y = sumy - rhsy;
      double tolx = jmax(0.0, sum_dvfbarL[k][0] - sum_Bpsi[k][0]);
      double toly = jmax(0.0, sum_dvfbarL[k][1] - sum_Bpsi[k][1]);
      std::vector<std::pair<double, int>> order(M);
      auto sort_desc = [&](const double* d) {
        for (int i = 0; i < M; ++i) order[i] = {d[i], i + 1};
        // sort!(..., rev=true) on (value, index) tuples: descending in isless order
        std::sort(order.begin(), order.end(), [](const std::pair<double, int>& a, const std::pair<double, int>& b) {
          if (jisless(b.first, a.first)) return true;
          if (jisless(a.first, b.first)) return false;
          return b.second < a.second;
        });
      };
      if (est_x > tolx) {
        sort_desc(dx);
        int curr = 1;
        double lhs = sumx;
        while (lhs > rhsx + tolx && curr <= M) {
          int idx = order[curr - 1].second;
          int si = ((idx - 1) % N1Dm1) + 1 + 1, sj = (idx - 1) / N1Dm1 + 1;  // 1-based
          double dvdf_v = dx[(si - 2) + N1Dm1 * (sj - 1)];
          if (dvdf_v < prm.ZEROTOL) break;
          lhs = lhs - Lx(si - 1, sj - 1) * dvdf_v;
          curr += 1;
        }
        for (int i = 1; i <= curr - 1; ++i) {
          int idx = order[i - 1].second;
          int si = ((idx - 1) % N1Dm1) + 1 + 1, sj = (idx - 1) / N1Dm1 + 1;
          double dvdf_v = dx[(si - 2) + N1Dm1 * (sj - 1)];
          double l_new = (i == curr - 1) ? jmax((rhsx + tolx - lhs) / dvdf_v, 0.0) : 0.0;
          Lx(si - 1, sj - 1) = jmin(Lx(si - 1, sj - 1), l_new);
        }
      }
      if (est_y > toly) {
        sort_desc(dy);
        int curr = 1;
        double lhs = sumy;
        while (lhs > rhsy + toly && curr <= M) {
          int idx = order[curr - 1].second;
          int si = ((idx - 1) % N1D) + 1, sj = (idx - 1) / N1D + 2;
          double dvdf_v = dy[(si - 1) + N1D * (sj - 2)];
          if (dvdf_v < prm.ZEROTOL) break;
          lhs = lhs - Ly(si - 1, sj - 1) * dvdf_v;
          curr += 1;
        }
        for (int i = 1; i <= curr - 1; ++i) {
          int idx = order[i - 1].second;
          int si = ((idx - 1) % N1D) + 1, sj = (idx - 1) / N1D + 2;
          double dvdf_v = dy[(si - 1) + N1D * (sj - 2)];
          double l_new = (i == curr - 1) ? jmax((rhsy + toly - lhs) / dvdf_v, 0.0) : 0.0;
          Ly(si - 1, sj - 1) = jmin(Ly(si - 1, sj - 1), l_new);
        }
      }
    }
  }

  // apply_rhs_limiter!(::ZhangShuLimiter) (limiter.jl:8-18), apply_zhang_shu_limiter!
  // (zhangshu.jl:4-25), zhang_shu_bound_limiter! (:35-45) with limiting_param
  // (::ZhangShuLimiter) (limiter_utils.jl:4-8): bounds (zeta rhoL, zeta rhoeL, Inf, Inf)
  std::vector<double> L_elem;  // L[k, nstage], K x Ns
  void apply_zhang_shu(double dt, int nstage) {
    const int s = nstage - 1;
    update_smoothness();
    const double zeta = prm.zeta;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < K; ++k) {
      double l = 1.0;
      for (int i = 0; i < Nq && !eq.kpp; ++i) {  // zhang_shu_bound_limiter!(::KPP): 1 (zhangshu.jl:58-60)
        const size_t ik = i + (size_t)Nq * k;
        const V4 uL = add(Uq[ik], scal(dt, rhsL[ik]));
        const V4 P = scal(dt, sub(rhsH[ik], rhsL[ik]));
        const double li = jmin(1.0, limiting_param_bound_rho_rhoe(uL, P, zeta * uL[0], zeta * eq.rhoe_ufun(uL), kInf, kInf));
        l = jmin(l, li);
      }
      L_elem[k + (size_t)K * s] = l;
      l = jmin(l, blending_factor[k]);
      for (int i = 0; i < Nq; ++i) {
        const size_t ik = i + (size_t)Nq * k;
        rhsU[ik] = add(scal(1 - l, rhsL[ik]), scal(l, rhsH[ik]));
      }
    }
  }

  // ---------------------------------------------------------------------------
  // rhs! (rhs.jl:5-13, 183-213)
  // ---------------------------------------------------------------------------
  double rhs(double t, double dt, int nstage) {
    // init_rhs! (rhs.jl:15-24): theta_local = 1, then the limiter's theta (filter.jl:1-16)
    std::fill(theta_local.begin() + (size_t)Nfp * K * (nstage - 1), theta_local.begin() + (size_t)Nfp * K * nstage, 1.0);
    if (gauss() && scaled_extrapolation()) solve_theta(nstage);
    switch (prm.rhs_type) {
      case P2DE_RHS_LOW_ORDER_POSITIVITY: {  // rhs.jl:183-189
        entropy_projection(nstage);
        double d = rhs_low_graph_visc(t, dt, nstage);
        rhsU = rhsL;
        return d;
      }
      case P2DE_RHS_ENTROPY_STABLE: {  // rhs.jl:191-197
        entropy_projection(nstage);
        rhs_fluxdiff(t, nstage);
        rhsU = rhsH;
        return dt;
      }
      default: {  // rhs.jl:199-213
        entropy_projection(nstage);
        double d = rhs_low_graph_visc(t, dt, nstage);
        rhs_fluxdiff(t, nstage);
        if (prm.rhs_limiter == P2DE_LIMITER_ZHANG_SHU) apply_zhang_shu(dt, nstage);
        else apply_rhs_limiter(t, dt, nstage);
        return d;
      }
    }
  }

  // SSP33! loop body (SSPRK33.jl:125-139)
  double ssp33_step(double& t) {
    const size_t n = Uq.size();
    double dt = jmin(prm.CFL * prm.dt0, prm.T - t);
#pragma omp parallel for schedule(static)
    for (size_t i = 0; i < n; ++i) resW[i] = Uq[i];
    dt = rhs(t, dt, 1);
#pragma omp parallel for schedule(static)
    for (size_t i = 0; i < n; ++i) Uq[i] = add(resW[i], scal(dt, rhsU[i]));
    rhs(t, dt, 2);
#pragma omp parallel for schedule(static)
    for (size_t i = 0; i < n; ++i) {
      resZ[i] = add(Uq[i], scal(dt, rhsU[i]));
      Uq[i] = add(scal(3.0 / 4.0, resW[i]), scal(1.0 / 4.0, resZ[i]));
    }
    rhs(t, dt, 3);
#pragma omp parallel for schedule(static)
    for (size_t i = 0; i < n; ++i) {
      resZ[i] = add(Uq[i], scal(dt, rhsU[i]));
      Uq[i] = add(scal(1.0 / 3.0, resW[i]), scal(2.0 / 3.0, resZ[i]));
    }
    t = t + dt;
    return dt;
  }
};

int validate(const p2de_param* p, const p2de_mesh* m, std::string& err) {
  if (!p || !m) {
    err = "null param or mesh";
    return P2DE_ERR_INVALID_ARGUMENT;
  }
  if (p->N < 1 || p->N > 7 || p->K < 1) {
    err = "N must be in 1..7 and K >= 1";
    return P2DE_ERR_INVALID_ARGUMENT;
  }
  if (!m->geom || !m->mapP) {
    err = "geom and mapP are required";
    return P2DE_ERR_INVALID_ARGUMENT;
  }
  if (p->approximation_basis < 0 || p->approximation_basis > 1 || p->entropyproj_limiter < 0 ||
      p->entropyproj_limiter > 1) {
    err = "approximation_basis and entropyproj_limiter must be 0 or 1";
    return P2DE_ERR_INVALID_ARGUMENT;
  }
  if (p->bound_type < 0 || p->bound_type > 9 || p->rhs_limiter < 0 || p->rhs_limiter > 1) {
    err = "bound_type must be in 0..9 and rhs_limiter in 0..1";
    return P2DE_ERR_INVALID_ARGUMENT;
  }
  if (p->equation < 0 || p->equation > 2) {
    err = "equation must be 0 (CompressibleEulerIdealGas{Dim2}), 1 (KPP) or 2 (CompressibleEulerIdealGas{Dim1})";
    return P2DE_ERR_INVALID_ARGUMENT;
  }
  if (p->equation == P2DE_EQUATION_COMPRESSIBLE_EULER_1D) {
    if (p->reference_semantics) {
      err = "CompressibleEulerIdealGas{Dim1}: the reference raises a MethodError in every RHS "
            "(Bx(::Dim1) calls reference_to_physical with dim last, rhs_utils.jl:18)";
      return P2DE_ERR_UNSUPPORTED;
    }
    if (m->nW || m->nS) {
      err = "CompressibleEulerIdealGas{Dim1}: periodic, inflow and outflow faces only";
      return P2DE_ERR_UNSUPPORTED;
    }
    const bool cell = p->bound_type == P2DE_BOUND_POSITIVITY_AND_CELL_ENTROPY || p->bound_type == P2DE_BOUND_TVD_AND_CELL_ENTROPY ||
                      p->bound_type == P2DE_BOUND_POSITIVITY_AND_RELAXED_CELL_ENTROPY ||
                      p->bound_type == P2DE_BOUND_TVD_AND_RELAXED_CELL_ENTROPY;
    if (cell && p->rhs_limiter == P2DE_LIMITER_SUBCELL && p->approximation_basis == P2DE_BASIS_GAUSS) {
      err = "CompressibleEulerIdealGas{Dim1}: no cell-entropy bounds on Gauss nodes "
            "(enforce_ES_subcell_interface! has no Dim1 method for GaussCollocation, subcell.jl:755-759)";
      return P2DE_ERR_UNSUPPORTED;
    }
  }
  if (p->equation == P2DE_EQUATION_KPP &&
      (p->approximation_basis != P2DE_BASIS_LOBATTO || m->nI || m->nO || m->nW || m->nS ||
       (p->rhs_limiter == P2DE_LIMITER_SUBCELL && p->bound_type != P2DE_BOUND_POSITIVITY))) {
    err = "KPP: LGL nodes, periodic or self-connected faces, PositivityBound or ZhangShu";
    return P2DE_ERR_UNSUPPORTED;
  }
  if ((p->low_order_surface_flux != P2DE_FLUX_LAX_FRIEDRICHS_ON_NODAL_VAL &&
       p->low_order_surface_flux != P2DE_FLUX_LAX_FRIEDRICHS_ON_PROJECTED_VAL) ||
      p->high_order_surface_flux != P2DE_FLUX_LAX_FRIEDRICHS_ON_PROJECTED_VAL) {
    err = "only LaxFriedrichsOnNodalVal (low) and LaxFriedrichsOnProjectedVal (high) surface fluxes";
    return P2DE_ERR_UNSUPPORTED;
  }
  return P2DE_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
// C API of the oracle (same descriptors as include/p2de.h)
// ---------------------------------------------------------------------------
extern "C" {

struct oracle_solver {
  Solver s;
};

int oracle_create(const p2de_param* prm, const p2de_mesh* mesh, int nthreads, oracle_solver** out) {
  std::string err;
  int st = validate(prm, mesh, err);
  if (st != P2DE_OK) {
    std::fprintf(stderr, "oracle_create: %s\n", err.c_str());
    return st;
  }
  auto* o = new oracle_solver();
  Solver& s = o->s;
  s.prm = *prm;
  s.N = prm->N;
  s.K = prm->K;
  s.eq.gamma = prm->gamma;
  s.eq.kpp = prm->equation == P2DE_EQUATION_KPP;
  s.dim1 = prm->equation == P2DE_EQUATION_COMPRESSIBLE_EULER_1D;
  s.Nd = s.dim1 ? 1 : 2;
  s.nthreads = nthreads;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
  s.build_operators();
  s.allocate();
  const int K = s.K, Nq = s.Nq, Nh = s.Nh, Nfp = s.Nfp;
  s.Jq.assign((size_t)Nq * K, 0.0);
  s.rxJh.assign((size_t)Nh * K, 0.0);
  s.sxJh = s.rxJh;
  s.ryJh = s.rxJh;
  s.syJh = s.rxJh;
  for (int k = 0; k < K; ++k) {
    const double* g = mesh->geom + 5 * (size_t)k;
    for (int i = 0; i < Nq; ++i) s.Jq[i + (size_t)Nq * k] = g[0];
    for (int i = 0; i < Nh; ++i) {
      size_t h = i + (size_t)Nh * k;
      s.rxJh[h] = g[1];
      s.sxJh[h] = g[2];
      s.ryJh[h] = g[3];
      s.syJh[h] = g[4];
    }
  }
  s.mapP.assign(mesh->mapP, mesh->mapP + (size_t)Nfp * K);
  if (mesh->nI > 0) {
    s.mapI.assign(mesh->mapI, mesh->mapI + mesh->nI);
    s.Ival.resize(mesh->nI);
    for (int64_t i = 0; i < mesh->nI; ++i) {
      if (s.dim1)  // (rho, rhou, E)
        s.Ival[i] = {mesh->Ival[3 * i], mesh->Ival[3 * i + 1], 0.0, mesh->Ival[3 * i + 2]};
      else
        for (int c = 0; c < 4; ++c) s.Ival[i][c] = mesh->Ival[4 * i + c];
    }
  }
  if (mesh->nO > 0) s.mapO.assign(mesh->mapO, mesh->mapO + mesh->nO);
  if (mesh->nW > 0) s.mapW.assign(mesh->mapW, mesh->mapW + mesh->nW);
  if (mesh->nS > 0) {
    s.mapS.assign(mesh->mapS, mesh->mapS + mesh->nS);
    s.xyS.assign(mesh->xyS, mesh->xyS + 2 * mesh->nS);
  }
  s.shock_x0 = mesh->shock_x0;
  s.shock_inv_slope = mesh->shock_inv_slope;
  s.shock_speed = mesh->shock_speed;
  for (int c = 0; c < 4; ++c) {
    s.shock_post[c] = mesh->shock_post[c];
    s.shock_pre[c] = mesh->shock_pre[c];
  }
  *out = o;
  return P2DE_OK;
}

int oracle_destroy(oracle_solver* o) {
  delete o;
  return P2DE_OK;
}

int oracle_set_Uq(oracle_solver* o, const double* Uq) {
  if (o->s.eq.kpp) {  // one component per node
    for (size_t i = 0; i < o->s.Uq.size(); ++i) o->s.Uq[i] = {Uq[i], 0.0, 0.0, 0.0};
    return P2DE_OK;
  }
  if (o->s.dim1) {  // (rho, rhou, E) per node
    for (size_t i = 0; i < o->s.Uq.size(); ++i) o->s.Uq[i] = {Uq[3 * i], Uq[3 * i + 1], 0.0, Uq[3 * i + 2]};
    return P2DE_OK;
  }
  std::memcpy(o->s.Uq.data(), Uq, sizeof(double) * 4 * o->s.Uq.size());
  return P2DE_OK;
}

int oracle_rhs(oracle_solver* o, double t, double dt, int nstage, double* dt_out) {
  if (nstage < 1 || nstage > 3) return P2DE_ERR_INVALID_ARGUMENT;
  *dt_out = o->s.rhs(t, dt, nstage);
  return P2DE_OK;
}

int oracle_ssp33_step(oracle_solver* o, double* t, double* dt_out) {
  *dt_out = o->s.ssp33_step(*t);
  return P2DE_OK;
}

int oracle_ssp33(oracle_solver* o, double* t_out, int64_t* steps, double* dt_last) {
  double t = o->s.prm.t0, dt = 0.0;
  int64_t n = 0;
  while (t < o->s.prm.T) {
    dt = o->s.ssp33_step(t);
    ++n;
    if (!(dt > 0.0)) break;
  }
  *t_out = t;
  *steps = n;
  *dt_last = dt;
  return P2DE_OK;
}

int oracle_get_field(oracle_solver* o, int field, int nstage, double* out) {
  Solver& s = o->s;
  const bool kpp = s.eq.kpp;  // KPP: component 0 of each state, (x, y) of each flux pair
  const bool d1 = s.dim1;     // Dim1: (rho, rhou, E) of each state, of the x part of each pair
  auto put3 = [&](size_t i, const V4& u) {
    out[3 * i] = u[0];
    out[3 * i + 1] = u[1];
    out[3 * i + 2] = u[3];
  };
  auto cp4 = [&](const std::vector<V4>& a) {
    if (d1)
      for (size_t i = 0; i < a.size(); ++i) put3(i, a[i]);
    else if (kpp)
      for (size_t i = 0; i < a.size(); ++i) out[i] = a[i][0];
    else
      std::memcpy(out, a.data(), sizeof(double) * 4 * a.size());
  };
  auto cp8 = [&](const std::vector<V2x4>& a) {
    if (d1)
      for (size_t i = 0; i < a.size(); ++i) put3(i, a[i].x);
    else if (kpp)
      for (size_t i = 0; i < a.size(); ++i) {
        out[2 * i] = a[i].x[0];
        out[2 * i + 1] = a[i].y[0];
      }
    else
      std::memcpy(out, a.data(), sizeof(double) * 8 * a.size());
  };
  switch (field) {
    case P2DE_FIELD_UQ: cp4(s.Uq); break;
    case P2DE_FIELD_RHSU: cp4(s.rhsU); break;
    case P2DE_FIELD_RHSL: cp4(s.rhsL); break;
    case P2DE_FIELD_RHSH: cp4(s.rhsH); break;
    case P2DE_FIELD_RHSXYL: cp8(s.rhsxyL); break;
    case P2DE_FIELD_RHSXYH: cp8(s.rhsxyH); break;
    case P2DE_FIELD_BF_L: cp8(s.BF_L); break;
    case P2DE_FIELD_BF_H: cp8(s.BF_H); break;
    case P2DE_FIELD_L_LOCAL: {
      if (nstage < 1 || nstage > 3) return P2DE_ERR_INVALID_ARGUMENT;
      size_t n = (size_t)(s.Nq + s.N1D) * s.Nd * s.K;
      std::memcpy(out, s.L_local.data() + n * (nstage - 1), sizeof(double) * n);
      break;
    }
    case P2DE_FIELD_RESW: cp4(s.resW); break;
    case P2DE_FIELD_L: {
      if (nstage < 1 || nstage > 3) return P2DE_ERR_INVALID_ARGUMENT;
      std::memcpy(out, s.L_elem.data() + (size_t)s.K * (nstage - 1), sizeof(double) * s.K);
      break;
    }
    case P2DE_FIELD_THETA_LOCAL: {
      if (nstage < 1 || nstage > 3) return P2DE_ERR_INVALID_ARGUMENT;
      size_t n = (size_t)s.Nfp * s.K;
      std::memcpy(out, s.theta_local.data() + n * (nstage - 1), sizeof(double) * n);
      break;
    }
    case P2DE_FIELD_F_BAR_H:
    case P2DE_FIELD_F_BAR_L: {  // f_bar[1] then f_bar[2], each (Nq+N1D) x K (Dim1: f_bar[1] only)
      const auto& fb = field == P2DE_FIELD_F_BAR_H ? s.f_bar_H : s.f_bar_L;
      const size_t n = fb[0].size();
      for (int d = 0; d < s.Nd; ++d) {
        if (fb[d].size() != n) return P2DE_ERR_INVALID_ARGUMENT;
        double* o = out + (size_t)d * n * (d1 ? 3 : kpp ? 1 : 4);
        for (size_t i = 0; i < n; ++i) {
          if (d1) {
            o[3 * i] = fb[d][i][0];
            o[3 * i + 1] = fb[d][i][1];
            o[3 * i + 2] = fb[d][i][3];
          } else if (kpp) {
            o[i] = fb[d][i][0];
          } else {
            for (int c = 0; c < 4; ++c) o[4 * i + c] = fb[d][i][c];
          }
        }
      }
      break;
    }
    default: return P2DE_ERR_INVALID_ARGUMENT;
  }
  return P2DE_OK;
}

// Operator data for the invariant tests: which = 0 r1D, 1 w1D, 2 D1D (row-major),
// 3 Srh_db (col-major Nh x Nh), 4 Ssh_db, 5 Sr0 (Nq x Nq), 6 Ss0, 7 wq.
int oracle_get_operator(oracle_solver* o, int which, double* out, int64_t* count) {
  Solver& s = o->s;
  const std::vector<double>* v = nullptr;
  switch (which) {
    case 0: v = &s.r1D; break;
    case 1: v = &s.w1D; break;
    case 2: v = &s.D1D; break;
    case 3: v = &s.Srh_db; break;
    case 4: v = &s.Ssh_db; break;
    case 5: v = &s.Sr0; break;
    case 6: v = &s.Ss0; break;
    case 7: v = &s.wq; break;
    default: return P2DE_ERR_INVALID_ARGUMENT;
  }
  *count = (int64_t)v->size();
  if (out) std::memcpy(out, v->data(), sizeof(double) * v->size());
  return P2DE_OK;
}

int oracle_nnz_counts(oracle_solver* o, int64_t* n_high, int64_t* n_low) {
  *n_high = (int64_t)o->s.Srsh_nnz.size();
  *n_low = (int64_t)o->s.Srs0_nnz.size();
  return P2DE_OK;
}

// Physics kernels for the unit tests.
int oracle_fS(double gamma, const double* UL6, const double* UR6, double* out8) {
  Euler e{gamma};
  V2x4 F = e.fS(UL6, UR6);
  for (int c = 0; c < 4; ++c) {
    out8[c] = F.x[c];
    out8[4 + c] = F.y[c];
  }
  return P2DE_OK;
}

int oracle_fluxes(double gamma, const double* U4, double* out8) {
  Euler e{gamma};
  V4 U{U4[0], U4[1], U4[2], U4[3]};
  V2x4 F = e.fluxes(U);
  for (int c = 0; c < 4; ++c) {
    out8[c] = F.x[c];
    out8[4 + c] = F.y[c];
  }
  return P2DE_OK;
}

double oracle_logmean(double aL, double aR) { return Euler::logmean(aL, aR, std::log(aL), std::log(aR)); }

int oracle_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // extern "C"
