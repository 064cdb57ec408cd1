// CompressibleEulerIdealGas{Dim1} on a Line mesh: P2DE.jl's RHS (rhs.jl:183-213) of the
// LimitedDG / LowOrderPositivity / FluxDiffRHS dispatches with the Dim1 methods of the
// subcell limiter (subcell.jl) or the Zhang-Shu limiter (zhangshu.jl), and the SSP-RK3
// stage update (SSPRK33.jl:125-139).
//
// One thread per element (per face node in the projection, per nonzero pair for the volume
// two-point terms). The kernels are written for agreement with the FP64 restatement: this
// translation unit is compiled without FMA contraction (-fmad=false) and keeps the
// reference's association order, so away from limiter decisions the results differ only
// through the last bits of log, exp and pow.
//
// States keep four slots per node, (rho, rhou, 0, E): with the y momentum 0 every Dim2
// point function below gives the Dim1 value of compressible_Navier_Stokes.jl exactly.
// Kernels of one stage: begin (dt) -> face projection -> low order (+ CFL) -> [initial
// min phi] -> volume pair terms -> high order + limiter factors -> symmetrization, limited
// fluxes, RK update; a step ends with t += dt on the device and is captured as one graph.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>

#include "p2de_args.h"
#include "p2de_line.h"
#include "p2de_physics.cuh"

namespace p2de {

namespace {

enum : int {
  LF_LOW = 1 << 0,         // low-order RHS
  LF_HIGH = 1 << 1,        // high-order RHS
  LF_SUBCELL = 1 << 2,     // SubcellLimiter
  LF_ZS = 1 << 3,          // ZhangShuLimiter
  LF_RHSU_L = 1 << 4,      // rhsU = rhsL (LowOrderPositivity)
  LF_RHSU_H = 1 << 5,      // rhsU = rhsH (FluxDiffRHS)
  LF_CFL = 1 << 6,         // stage 1 of a low-order RHS: the positivity CFL
  LF_LFPROJ = 1 << 7,      // LaxFriedrichsOnProjectedVal low-order flux
  LF_NSE = 1 << 8,         // NodewiseScaledExtrapolation on Gauss nodes
  LF_SHOCK = 1 << 9,       // HennemannShockCapture
  LF_TVD = 1 << 10,        // TVD density bounds
  LF_MINENT = 1 << 11,     // min-entropy bound
  LF_RELAXED = 1 << 12,    // relaxed bounds (smoothness factor)
  LF_CELL = 1 << 13,       // cell-entropy bound
  LF_UPDATE = 1 << 14,     // RK stage update of Uq
};

// One warp per block: a block's warps share their SM's FP64 pipe, which issues a warp
// instruction in the same time however many lanes it carries, so a small solve is fastest
// with its elements spread one warp per SM (32-thread blocks still fill an SM at large K).
constexpr int kThreads = 32;
// The team layout (P2DE_LAYOUT_TEAM): kTeam lanes per element, kTeamE elements per one-warp
// block, for solves too small to fill the GPU one thread per element; a Line solve starts with
// it below kTeamMaxK elements. The team kernels trade total work for a shorter chain per
// element (the speculative bisection evaluates 155 midpoints per face node where the loop
// evaluates 22), so they win only while the GPU is idle: Shu-Osher data, N = 3, ms per step
// one thread per element / team: K = 1024 1.35 / 0.70, K = 4096 1.40 / 1.88, K = 8192
// 1.40 / 3.64.
constexpr int kTeam = 16;
constexpr int kTeamE = 32 / kTeam;
constexpr int kTeamMaxK = 2048;
constexpr int MQ = kMaxN1D;     // nodes per element at most
constexpr int MH = kLineMaxNh;  // nodes + face nodes
constexpr int MS = 2 * kMaxN1D; // rows of L_local
// the device-resident time state of a solve
enum : int { TS_T = 0, TS_DT = 1, TS_DONE = 2, TS_STEPS = 3, TS_PHI = 4, TS_N = 8 };

struct LineArgs {
  int K, N1D, nstage, flags;
  const LineOps* ops;
  double *Uq, *resW, *rhsL, *rhsH, *rhsU, *BFL, *BFH, *uf, *theta, *Lloc, *Lraw, *fbar, *Lelem, *sf;
  const double *geom, *Ival;
  long long* phikey;
  const int32_t *nbr, *bcidx;
  const int8_t* bc;
  unsigned long long* dtkey;
  long long* minrec;
  int* status;
  double* ts;  // TS_* slots
  double gamma, POSTOL, ZEROTOL, zeta, eta, CFL, beta, sc_TN, sc_sfac, s0, T, dt0, t0;
};

// a finished time loop turns every later launch of the step into a no-op
__device__ __forceinline__ bool done(const LineArgs& a) { return a.ts[TS_DONE] != 0.0; }

// ---- point functions (compressible_Navier_Stokes.jl; four slots, y momentum 0) ----------
__device__ double pfun4(double gamma, const double* U) {
  return (gamma - 1.0) * (U[3] - 0.5 * (U[1] * U[1] + U[2] * U[2]) / U[0]);
}
__device__ double rhoe4(const double* U) { return U[3] - 0.5 * (U[1] * U[1] + U[2] * U[2]) / U[0]; }
__device__ double betafun4(double gamma, const double* U) { return U[0] / (2.0 * pfun4(gamma, U)); }
// wavespeed_estimate(::Dim1) (:48-52) of (rho, un, E)
__device__ double wavespeed1(double gamma, double rho, double rhou, double E) {
  const double p = (gamma - 1.0) * (E - 0.5 * (rhou * rhou) / rho);
  return fabs(rhou / rho) + sqrt(gamma * p / rho);
}
__device__ double wavespeed4(double gamma, const double* U, double n1, double n2) {
  return wavespeed1(gamma, U[0], n1 * U[1] + n2 * U[2], U[3]);
}
__device__ void fluxes4(double gamma, const double* U, double* f) {  // the x flux
  const double rho = U[0], rhou = U[1], rhov = U[2], E = U[3];
  const double p = pfun4(gamma, U);
  const double u = rhou / rho, v = rhov / rho;
  f[0] = rhou;
  f[1] = rhou * u + p;
  f[2] = rho * u * v;
  f[3] = u * (E + p);
}
__device__ void v_ufun4(double gamma, const double* U, double* V) {
  const double p = pfun4(gamma, U);
  const double s = log(p / pow(U[0], gamma));
  V[0] = (gamma + 1.0 - s) - (gamma - 1.0) * U[3] / p;
  V[1] = U[1] * (gamma - 1.0) / p;
  V[2] = U[2] * (gamma - 1.0) / p;
  V[3] = -U[0] * (gamma - 1.0) / p;
}
__device__ void u_vfun4(double gamma, const double* V, double* U) {
  const double s = gamma - V[0] + (V[1] * V[1] + V[2] * V[2]) / (2.0 * V[3]);
  const double rhoeV = pow((gamma - 1.0) / pow(-V[3], gamma), 1.0 / (gamma - 1.0)) * exp(-s / (gamma - 1.0));
  U[0] = -rhoeV * V[3];
  U[1] = rhoeV * V[1];
  U[2] = rhoeV * V[2];
  U[3] = rhoeV * (1.0 - (V[1] * V[1] + V[2] * V[2]) / (2.0 * V[3]));
}
// logmean (:307-321)
__device__ double logmean(double aL, double aR, double logL, double logR) {
  const double da = aR - aL, aavg = 0.5 * (aR + aL);
  const double f = da / aavg, v = f * f;
  if (fabs(f) < 1e-4) return aavg * (1.0 + v * (-0.2 - v * (0.0512 - v * 0.026038857142857)));
  return -da / (logL - logR);
}
// fS (:196-218) as the Dim2 x flux with v = 0; U = (rho, u, v, beta, log rho, log beta)
__device__ void fS4(double gamma, const double* UL, const double* UR, double* F) {
  const double rholog = logmean(UL[0], UR[0], UL[4], UR[4]);
  const double betalog = logmean(UL[3], UR[3], UL[5], UR[5]);
  const double rhoavg = 0.5 * (UL[0] + UR[0]);
  const double uavg = 0.5 * (UL[1] + UR[1]);
  const double vavg = 0.5 * (UL[2] + UR[2]);
  const double unorm = UL[1] * UR[1] + UL[2] * UR[2];
  const double pa = rhoavg / (UL[3] + UR[3]);
  const double f4aux = rholog / (2.0 * (gamma - 1.0) * betalog) + pa + 0.5 * rholog * unorm;
  const double FxS1 = rholog * uavg;
  F[0] = FxS1;
  F[1] = FxS1 * uavg + pa;
  F[2] = FxS1 * vavg;
  F[3] = f4aux * uavg;
}
__device__ double s_modified4(double gamma, const double* U) { return rhoe4(U) * pow(U[0], -gamma); }
// isless on Float64 (NaN last, -0.0 before 0.0)
__device__ bool jisless(double a, double b) {
  if (isnan(a)) return false;
  if (isnan(b)) return true;
  if (a < b) return true;
  if (a == b) return signbit(a) && !signbit(b);
  return false;
}
__device__ double decode_key(long long k) { return __longlong_as_double(k ^ ((k >> 63) & 0x7fffffffffffffffLL)); }
__device__ long long encode_key(double x) {
  const long long b = __double_as_longlong(x);
  return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}

// ---- limiter helpers (limiter_utils.jl) ----------------------------------------------
// :108-132 with the coefficients of :141-146
__device__ double rhoe_quadratic_solve(const double* U, const double* P, double Lrhoe, double ZEROTOL) {
  if (Lrhoe == INFINITY) return 1.0;
  const double a = P[0] * P[3] - 1.0 / 2.0 * (P[1] * P[1] + P[2] * P[2]);
  const double b = U[3] * P[0] + U[0] * P[3] - U[1] * P[1] - U[2] * P[2] - P[0] * Lrhoe;
  const double c = U[3] * U[0] - 1.0 / 2.0 * (U[1] * U[1] + U[2] * U[2]) - U[0] * Lrhoe;
  double l = 1.0;
  if (b * b - 4.0 * a * c >= 0.0) {
    const double r1 = (-b + sqrt(b * b - 4.0 * a * c)) / (2.0 * a);
    const double r2 = (-b - sqrt(b * b - 4.0 * a * c)) / (2.0 * a);
    if (r1 > ZEROTOL && r2 > ZEROTOL)
      l = jmin(r1, r2);
    else if (r1 > ZEROTOL && r2 < -ZEROTOL)
      l = r1;
    else if (r2 > ZEROTOL && r1 < -ZEROTOL)
      l = r2;
  }
  return l;
}
// :82-96
__device__ double bound_rho_rhoe(const double* U, const double* P, double Lrho, double Lrhoe, double Urho,
                                 double Urhoe, double ZEROTOL) {
  double l = 1.0;
  if (U[0] + P[0] < Lrho) l = jmax((Lrho - U[0]) / P[0], 0.0);
  if (U[0] + P[0] > Urho) l = jmin(l, jmax((Urho - U[0]) / P[0], 0.0));
  return jmin(jmin(l, rhoe_quadratic_solve(U, P, Lrhoe, ZEROTOL)), rhoe_quadratic_solve(U, P, Urhoe, ZEROTOL));
}
// find_alpha (low_order_graph_viscosity.jl:316-345), the doubling bounded
__device__ double find_alpha(const double* ui, const double* ut, double POSTOL) {
  auto ok = [&](double al) {
    double q[4];
    for (int c = 0; c < 4; ++c) q[c] = al * ui[c] - ut[c];
    return q[0] > POSTOL && rhoe4(q) > POSTOL;
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

__device__ void ld4(const double* p, double* u) {
  for (int c = 0; c < 4; ++c) u[c] = p[c];
}
__device__ void st4(double* p, const double* u) {
  for (int c = 0; c < 4; ++c) p[c] = u[c];
}

// Face state of the element's own low-order flux: the projected face value
// (LaxFriedrichsOnProjectedVal) or the face node's value (LaxFriedrichsOnNodalVal)
__device__ void low_face_state(const LineArgs& a, int k, int f, double* u) {
  const int N = a.N1D - 1;
  if (a.flags & LF_LFPROJ)
    ld4(a.uf + 4 * (2 * (size_t)k + f), u);
  else
    ld4(a.Uq + 4 * ((size_t)a.N1D * k + (f == 0 ? 0 : N)), u);
}

// Bx (rhs_utils.jl:13-19) with the Dim2 reference_to_physical of geometry (J, rxJ, sxJ, ryJ, syJ)
__device__ void Bx(const LineArgs& a, int k, int f, double& b0, double& b1) {
  const double* g = a.geom + 5 * (size_t)k;
  const double Br = a.ops->rxf[f], Bs = 0.0;
  b0 = g[1] * Br + g[2] * Bs;
  b1 = g[3] * Br + g[4] * Bs;
}
__device__ double norm2(double x, double y) {
  const double m = fmax(fabs(x), fabs(y));
  if (m == 0.0 || isinf(m) || isnan(m)) return m;
  return sqrt(x * x + y * y);
}

// smoothness indicator (shock_capture.jl:14-45), blending factor (:118-137) and smoothness
// factor (subcell.jl:927-956) of element k
__device__ void smoothness(const LineArgs& a, const double (*U)[4], double& blend, double& epsk) {
  const int n = a.N1D, N = n - 1;
  const bool need = (a.flags & (LF_SHOCK | LF_RELAXED)) != 0;
  double ind = 0.0;
  if (need) {
    double iv[MQ];
    for (int i = 0; i < n; ++i) iv[i] = U[i][0] * pfun4(a.gamma, U[i]);
    double modeN = 0.0, modeNm1 = 0.0, total = 0.0;
    for (int i = 0; i <= N; ++i) {
      double m = 0.0;
      for (int j = 0; j < n; ++j) m += a.ops->VDMinv[i * n + j] * iv[j];
      const double energy = m * m;
      if (i == N) modeN += energy;
      if (i == N - 1) modeNm1 += energy;
      total += energy;
    }
    ind = jmax(modeN / total, modeNm1 / total);
  }
  blend = 1.0;
  if (a.flags & LF_SHOCK) {
    const double alpha = 1.0 / (1.0 + exp(-a.sc_sfac / a.sc_TN * (ind - a.sc_TN)));
    blend = jmax(jmin(1.0 - alpha, 1.0), 0.5);
  }
  epsk = (a.flags & LF_MINENT) ? 1.0 : 0.0;
  if (a.flags & LF_RELAXED) {
    const double kappa = 1.0;
    const double sk = log(ind) / 2.302585092994046;  // log(10), correctly rounded
    if (sk < a.s0 - kappa)
      epsk = 0.0;
    else if (sk > a.s0 + kappa)
      epsk = 1.0;
    else
      epsk = 0.5 - 0.5 * sin(3.141592653589793 * (sk - a.s0) / (2 * kappa));
  }
}

// ---- kernels ----------------------------------------------------------------------------
// stage begin. dtkey[0]: the step's dt (lowered by the stage-1 CFL), dtkey[1]: the stage's
// TimeParam dt, which the limiter reads (at stage 1 the dt before the CFL, rhs.jl:41-55 with
// SSPRK33.jl:30-37). mode 0 (a lone RHS): (dt, dt_lim) from the host, phi reset as given;
// mode 1 (stages 2, 3 of a step): dtkey[1] = dtkey[0]; mode 2 (stage 1 of a step): from the
// device time t, the loop's end test (SSPRK33.jl:29), dt = min(CFL dt0, T - t) for both,
// the stage minima reset, and the initial min of phi reset when t == t0 (subcell.jl:31-34).
__global__ void k_line_begin(LineArgs a, int mode, double dt, double dt_lim, int phi) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  if (mode == 1) {
    a.dtkey[1] = a.dtkey[0];
    return;
  }
  if (mode == 2) {
    const double t = a.ts[TS_T];
    if (!(t < a.T)) {
      a.ts[TS_DONE] = 1.0;
      return;
    }
    dt = dt_lim = jmin(a.CFL * a.dt0, a.T - t);
    phi = phi && t == a.t0;
  }
  a.ts[TS_DONE] = 0.0;
  a.ts[TS_PHI] = phi ? 1.0 : 0.0;
  a.dtkey[0] = (unsigned long long)__double_as_longlong(dt);
  a.dtkey[1] = (unsigned long long)__double_as_longlong(dt_lim);
  for (int i = 0; i < 6; ++i) a.minrec[i] = encode_key(INFINITY);
  if (phi) *a.phikey = encode_key(INFINITY);
}

// step end (SSPRK33.jl:38-39): t += dt, the step count
__global__ void k_line_end(LineArgs a) {
  if (threadIdx.x != 0 || blockIdx.x != 0 || done(a)) return;
  const double dt = __longlong_as_double((long long)a.dtkey[0]);
  a.ts[TS_T] = a.ts[TS_T] + dt;
  a.ts[TS_DT] = dt;
  a.ts[TS_STEPS] = a.ts[TS_STEPS] + 1.0;
}

// entropy_projection! (rhs.jl:59-133) with solve_theta!(::NodewiseScaledExtrapolation)
// (filter.jl:6-62, 91-130) on Gauss nodes: theta_local and the projected face states. One
// thread per face node (the two bisections of an element run side by side).
template <int NQ>
__global__ void k_line_face(LineArgs a) {
  const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= 2LL * a.K || done(a)) return;
  const int k = (int)(g / 2), f = (int)(g % 2);
  constexpr int n = NQ, N = n - 1;
  const int s = a.nstage - 1;
  const LineOps& o = *a.ops;
  double U[MQ][4], v[MQ][4];
  for (int i = 0; i < n; ++i) {
    ld4(a.Uq + 4 * ((size_t)n * k + i), U[i]);
    v_ufun4(a.gamma, U[i], v[i]);
  }
  {
    const int fn = f == 0 ? 0 : N;
    auto face_var = [&](double th, double* acc) {
      for (int c = 0; c < 4; ++c) acc[c] = 0.0;
      for (int j = 0; j < n; ++j) {
        const double c = th * o.Vf[f][j] + (1.0 - th) * (j == fn ? 1.0 : 0.0);
        for (int q = 0; q < 4; ++q) acc[q] = acc[q] + c * v[j][q];
      }
    };
    double th = 1.0;
    if (a.flags & LF_NSE) {
      double Ufv[4] = {0, 0, 0, 0}, VUf[4] = {0, 0, 0, 0};
      for (int j = 0; j < n; ++j)
        for (int q = 0; q < 4; ++q) {
          Ufv[q] = Ufv[q] + o.Vf[f][j] * U[j][q];
          VUf[q] = VUf[q] + o.Vf[f][j] * v[j][q];
        }
      const double rhoef = rhoe4(Ufv), eps = a.POSTOL, zeta = a.zeta, eta = a.eta;
      auto ok = [&](double t) {
        double vt[4], ut[4];
        face_var(t, vt);
        if (!(vt[3] < -eps)) return false;
        u_vfun4(a.gamma, vt, ut);
        const double rho = ut[0], re = rhoe4(ut);
        return vt[3] < jmin(zeta * VUf[3], -eps) && rho > jmax((1 - eta) * Ufv[0], eps) && rho < (1 + eta) * Ufv[0] &&
               re > jmax((1 - eta) * rhoef, eps) && re < (1 + eta) * rhoef;
      };
      double x_valid = 0.0, x_invalid = 1.0;
      if (ok(x_invalid)) {
        th = x_invalid;
      } else {
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
    a.theta[2 * ((size_t)a.K * s + k) + f] = th;
    double acc[4], u[4];
    face_var(th, acc);
    u_vfun4(a.gamma, acc, u);
    st4(a.uf + 4 * (2 * (size_t)k + f), u);
  }
}

// k_line_face with one warp per face node (two per element, a block of 64 threads). The
// entropy variables of the nodes are formed once per element (one lane per node), and the
// bisection of solve_theta! runs speculatively: each round, lanes 1..31 of a warp evaluate
// the 31 midpoints of the next five levels of the bisection tree below the current interval
// (lane j replays the midpoints on the path to heap node j, the very operations the
// sequential bisection performs on that path), and the warp walks the tree with a ballot of
// the results. The 21 halvings take five rounds, the first one with lane 0 testing theta = 1.
// The projected face state at the final theta is the one the test of that theta formed on
// its lane (the same face_var and u_vfun4 of the same theta), passed by a shuffle; it is
// formed anew only when no test passed (theta = 0). theta and the projected face state are
// the bits of the one-thread kernel.
constexpr int kFaceTeamThreads = 64;

template <int NQ>
__global__ void k_line_face_team(LineArgs a) {
  constexpr int n = NQ, N = n - 1, D = 5;  // tree levels per round: 2^D - 1 = 31 lanes
  const int k = blockIdx.x;
  if (k >= a.K || done(a)) return;  // the same for the whole block
  const int lane = threadIdx.x % 32, f = threadIdx.x / 32;
  const int s = a.nstage - 1;
  const LineOps& o = *a.ops;
  __shared__ double sU[n][4], sv[n][4];
  if (threadIdx.x < n) {
    ld4(a.Uq + 4 * ((size_t)n * k + threadIdx.x), sU[threadIdx.x]);
    v_ufun4(a.gamma, sU[threadIdx.x], sv[threadIdx.x]);
  }
  __syncthreads();
  const int fn = f == 0 ? 0 : N;
  auto face_var = [&](double th, double* acc) {
    for (int c = 0; c < 4; ++c) acc[c] = 0.0;
    for (int j = 0; j < n; ++j) {
      const double c = th * o.Vf[f][j] + (1.0 - th) * (j == fn ? 1.0 : 0.0);
      for (int q = 0; q < 4; ++q) acc[q] = acc[q] + c * sv[j][q];
    }
  };
  double th = 1.0;
  double u[4];
  bool have_u = false;  // u holds u_vfun(face_var(th)) (the same on every lane of the warp)
  if (a.flags & LF_NSE) {
    double Ufv[4] = {0, 0, 0, 0}, VUf[4] = {0, 0, 0, 0};
    for (int j = 0; j < n; ++j)
      for (int q = 0; q < 4; ++q) {
        Ufv[q] = Ufv[q] + o.Vf[f][j] * sU[j][q];
        VUf[q] = VUf[q] + o.Vf[f][j] * sv[j][q];
      }
    const double rhoef = rhoe4(Ufv), eps = a.POSTOL, zeta = a.zeta, eta = a.eta;
    // the test of solve_theta!; ut: the projected state it formed (when it got that far)
    auto ok = [&](double t, double* ut) {
      double vt[4];
      face_var(t, vt);
      if (!(vt[3] < -eps)) return false;
      u_vfun4(a.gamma, vt, ut);
      const double rho = ut[0], re = rhoe4(ut);
      return vt[3] < jmin(zeta * VUf[3], -eps) && rho > jmax((1 - eta) * Ufv[0], eps) && rho < (1 + eta) * Ufv[0] &&
             re > jmax((1 - eta) * rhoef, eps) && re < (1 + eta) * rhoef;
    };
    double x_valid = 0.0, x_invalid = 1.0;
    bool settled = false;  // theta = 1 passed
    int left = 21;         // halvings of the sequential loop (iter = 0..20)
    double ut[4] = {0, 0, 0, 0};
    // five rounds (5 + 5 + 5 + 5 + 1 levels); the branch conditions below are the same on
    // every lane of the warp (they depend on ballots only), so each shuffle is warp-uniform
    for (int round = 0; round < 5; ++round) {
      // lane j (1..31): the midpoint of heap node j below (x_valid, x_invalid); lane 0, in
      // the first round, tests theta = 1
      const int levels = left < D ? left : D;
      bool res = false;
      if (lane == 0) {
        if (round == 0) res = ok(x_invalid, ut);
      } else if (!settled && 31 - __clz(lane) < levels) {
        const int d = 31 - __clz(lane);  // depth of the heap node
        double xv = x_valid, xi = x_invalid;
        for (int l = 0; l < d; ++l) {
          const double mid = 0.5 * (xv + xi);
          if ((lane >> (d - 1 - l)) & 1)
            xv = mid;
          else
            xi = mid;
        }
        res = ok(0.5 * (xv + xi), ut);
      }
      const unsigned ball = __ballot_sync(0xffffffffu, res);
      int src = -1;  // the lane whose test set the warp's current x_valid (or passed theta = 1)
      if (round == 0 && (ball & 1u)) {
        settled = true;
        src = 0;
      }
      if (!settled) {
        int j = 1;
        for (int l = 0; l < levels; ++l) {
          const double x_new = 0.5 * (x_valid + x_invalid);
          const int r = (ball >> j) & 1;
          if (r) {
            x_valid = x_new;
            src = j;
          } else {
            x_invalid = x_new;
          }
          j = 2 * j + r;
        }
      }
      if (src >= 0) {
        for (int c = 0; c < 4; ++c) u[c] = __shfl_sync(0xffffffffu, ut[c], src);
        have_u = true;
      }
      left -= levels;
    }
    th = settled ? x_invalid : x_valid;
  }
  if (lane == 0) {
    a.theta[2 * ((size_t)a.K * s + k) + f] = th;
    if (!have_u) {
      double acc[4];
      face_var(th, acc);
      u_vfun4(a.gamma, acc, u);
    }
    st4(a.uf + 4 * (2 * (size_t)k + f), u);
  }
}

// rhs_low_graph_visc! (low_order_graph_viscosity.jl:4-41) with the Dim1 graph viscosity and
// LF placement (rhs_utils.jl:78-113); stage 1: the element's positivity CFL (:222-309)
template <int NQ>
__global__ void k_line_low(LineArgs a) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= a.K || done(a)) return;
  constexpr int n = NQ, N = n - 1;
  const LineOps& o = *a.ops;
  const double* g = a.geom + 5 * (size_t)k;
  const double J = g[0];
  double U[MQ][4], fl[MQ][4], r[MQ][4], lamR[MQ];
  for (int i = 0; i < n; ++i) {
    ld4(a.Uq + 4 * ((size_t)n * k + i), U[i]);
    fluxes4(a.gamma, U[i], fl[i]);
    for (int c = 0; c < 4; ++c) r[i][c] = 0.0;
    lamR[i] = 0.0;
  }
  // accumulate_low_order_rhs_volume! (:139-173): pairs (j+1, j), Sr0[j+1, j] = -1/2
  for (int j = 0; j < N; ++j) {
    const int i = j + 1;
    const double Sr0 = 0.5 * (-0.5 - 0.5), Ss0 = 0.0;
    const double S0 = g[1] * Sr0 + g[2] * Ss0, S1 = g[3] * Sr0 + g[4] * Ss0;
    const double nn = norm2(S0, S1), n1 = S0 / nn, n2 = S1 / nn;
    const double ws = jmax(wavespeed4(a.gamma, U[i], n1, n2), wavespeed4(a.gamma, U[j], -n1, -n2));
    const double lij = nn * ws;
    lamR[j] = lij;
    for (int c = 0; c < 4; ++c) {
      const double F = 0.5 * (fl[i][c] + fl[j][c]);
      const double SF = 2.0 * S0 * F - lij * (U[j][c] - U[i][c]);
      r[i][c] = r[i][c] + SF;  // Q0F1, negated below
      r[j][c] = r[j][c] + -SF;
    }
  }
  for (int i = 0; i < n; ++i)
    for (int c = 0; c < 4; ++c) r[i][c] = 0.0 - r[i][c];
  // accumulate_low_order_rhs_surface! (:175-204) with get_uP_and_enforce_BC! (:94-124)
  double lamB[2], wsf[2];
#pragma unroll
  for (int f = 0; f < 2; ++f) {
    const int fk = 2 * k + f, p = a.nbr[fk], kP = p / 2, iP = p % 2;
    double Uf[4], UfP[4], uP[4], b0, b1, bP0, bP1;
    low_face_state(a, k, f, Uf);
    low_face_state(a, kP, iP, UfP);
    Bx(a, k, f, b0, b1);
    Bx(a, kP, iP, bP0, bP1);
    const double nn = norm2(b0, b1), nnP = norm2(bP0, bP1);
    wsf[f] = wavespeed4(a.gamma, Uf, b0 / nn, b1 / nn);
    const double wsP = wavespeed4(a.gamma, UfP, bP0 / nnP, bP1 / nnP);
    const int8_t bc = a.bc[fk];
    if (bc == BC_INFLOW) {
      const double* I = a.Ival + 3 * (size_t)a.bcidx[fk];
      uP[0] = I[0], uP[1] = I[1], uP[2] = 0.0, uP[3] = I[2];
    } else if (bc == BC_OUTFLOW) {
      ld4(U[f == 0 ? 0 : N], uP);
    } else {
      ld4(UfP, uP);
    }
    lamB[f] = 0.5 * nn * jmax(wsf[f], wsP);
    double ff[4], fP[4];
    fluxes4(a.gamma, Uf, ff);
    fluxes4(a.gamma, uP, fP);
    double BF[4];
    for (int c = 0; c < 4; ++c) {
      const double fs = 0.5 * (ff[c] + fP[c]);
      BF[c] = b0 * fs - lamB[f] * (uP[c] - Uf[c]);
    }
    st4(a.BFL + 4 * (size_t)fk, BF);
    const int q = f == 0 ? 0 : N;
    for (int c = 0; c < 4; ++c) r[q][c] = r[q][c] - BF[c];
  }
  // scale_low_order_rhs_by_mass! (:206-220)
  for (int i = 0; i < n; ++i) {
    const double wJq = J * o.wq[i];
    double rl[4];
    for (int c = 0; c < 4; ++c) rl[c] = r[i][c] / wJq + 0.0;
    st4(a.rhsL + 4 * ((size_t)n * k + i), rl);
    if (a.flags & LF_RHSU_L) st4(a.rhsU + 4 * ((size_t)n * k + i), rl);
  }
  if (a.flags & LF_CFL) {
    double dtl = INFINITY;
    for (int i = 0; i < n; ++i) {
      double li = 0.0;
      for (int j = 0; j < n; ++j) li += (j == i - 1) ? lamR[j] : ((j == i + 1) ? lamR[i] : 0.0);
      if (i == 0 || i == N) {
        const int f = i == 0 ? 0 : 1;
        if (a.flags & LF_LFPROJ) {
          double b0, b1, ut[4];
          Bx(a, k, f, b0, b1);
          ld4(a.uf + 4 * (2 * (size_t)k + f), ut);
          li += find_alpha(U[i], ut, a.POSTOL) * lamB[f] + 0.5 * norm2(b0, b1) * wsf[f];
        } else {
          li += lamB[f];
        }
      }
      const double wJq = J * o.wq[i];
      dtl = jmin(dtl, a.CFL * 0.5 * wJq / li);
    }
    if (dtl > 0.0)
      atomicMin(&a.dtkey[0], (unsigned long long)__double_as_longlong(dtl));
    else
      atomicOr(a.status, ST_BAD_DT);
  }
}

// k_line_low with a team of kTeam lanes per element (kTeamE elements per one-warp block): the
// node fluxes, the N low-order pairs, the two faces and the nodes' mass scaling and CFL terms
// on separate lanes, each value formed by the same expression and in the same order as in
// k_line_low (same bits); the element's CFL minimum is taken in node order on the team's
// first lane.
template <int NQ>
__global__ void k_line_low_team(LineArgs a) {
  constexpr int n = NQ, N = n - 1, E = kTeamE;
  static_assert(n <= kTeam / 2, "pairs and faces on separate lanes");
  const int lane = threadIdx.x % kTeam, e = threadIdx.x / kTeam;
  const int k = blockIdx.x * E + e;
  if (done(a)) return;  // the same for the whole grid
  const bool live = k < a.K;
  const LineOps& o = *a.ops;
  __shared__ double sU[E][n][4], sfl[E][n][4], sSF[E][n][4], slamR[E][n], sBF[E][2][4], slamB[E][2], swsf[E][2];
  __shared__ double scand[E][n];
  double(*U)[4] = sU[e];
  double(*fl)[4] = sfl[e];
  double(*SF)[4] = sSF[e];
  double* lamR = slamR[e];
  double(*BF)[4] = sBF[e];
  double *lamB = slamB[e], *wsf = swsf[e];
  const double* g = live ? a.geom + 5 * (size_t)k : a.geom;
  const double J = g[0];
  if (live && lane < n) {
    ld4(a.Uq + 4 * ((size_t)n * k + lane), U[lane]);
    fluxes4(a.gamma, U[lane], fl[lane]);
    lamR[lane] = 0.0;
  }
  __syncwarp();
  // accumulate_low_order_rhs_volume! (:139-173): pair (j+1, j) on lane j, Sr0[j+1, j] = -1/2
  if (live && lane < N) {
    const int j = lane, i = j + 1;
    const double Sr0 = 0.5 * (-0.5 - 0.5), Ss0 = 0.0;
    const double S0 = g[1] * Sr0 + g[2] * Ss0, S1 = g[3] * Sr0 + g[4] * Ss0;
    const double nn = norm2(S0, S1), n1 = S0 / nn, n2 = S1 / nn;
    const double ws = jmax(wavespeed4(a.gamma, U[i], n1, n2), wavespeed4(a.gamma, U[j], -n1, -n2));
    const double lij = nn * ws;
    lamR[j] = lij;
    for (int c = 0; c < 4; ++c) {
      const double F = 0.5 * (fl[i][c] + fl[j][c]);
      SF[j][c] = 2.0 * S0 * F - lij * (U[j][c] - U[i][c]);
    }
  }
  // accumulate_low_order_rhs_surface! (:175-204) with get_uP_and_enforce_BC! (:94-124), face f
  // on lane kTeam/2 + f
  if (live && lane >= kTeam / 2 && lane < kTeam / 2 + 2) {
    const int f = lane - kTeam / 2;
    const int fk = 2 * k + f, p = a.nbr[fk], kP = p / 2, iP = p % 2;
    double Uf[4], UfP[4], uP[4], b0, b1, bP0, bP1;
    low_face_state(a, k, f, Uf);
    low_face_state(a, kP, iP, UfP);
    Bx(a, k, f, b0, b1);
    Bx(a, kP, iP, bP0, bP1);
    const double nn = norm2(b0, b1), nnP = norm2(bP0, bP1);
    wsf[f] = wavespeed4(a.gamma, Uf, b0 / nn, b1 / nn);
    const double wsP = wavespeed4(a.gamma, UfP, bP0 / nnP, bP1 / nnP);
    const int8_t bc = a.bc[fk];
    if (bc == BC_INFLOW) {
      const double* I = a.Ival + 3 * (size_t)a.bcidx[fk];
      uP[0] = I[0], uP[1] = I[1], uP[2] = 0.0, uP[3] = I[2];
    } else if (bc == BC_OUTFLOW) {
      ld4(U[f == 0 ? 0 : N], uP);
    } else {
      ld4(UfP, uP);
    }
    lamB[f] = 0.5 * nn * jmax(wsf[f], wsP);
    double ff[4], fP[4];
    fluxes4(a.gamma, Uf, ff);
    fluxes4(a.gamma, uP, fP);
    for (int c = 0; c < 4; ++c) {
      const double fs = 0.5 * (ff[c] + fP[c]);
      BF[f][c] = b0 * fs - lamB[f] * (uP[c] - Uf[c]);
    }
    st4(a.BFL + 4 * (size_t)fk, BF[f]);
  }
  __syncwarp();
  // per node: Q0F1 in pair order (+SF of pair m-1, then -SF of pair m), negated, the face
  // term, scale_low_order_rhs_by_mass! (:206-220) and the node's CFL term (:222-309)
  if (live && lane < n) {
    const int m = lane;
    double r[4] = {0.0, 0.0, 0.0, 0.0};
    if (m >= 1)
      for (int c = 0; c < 4; ++c) r[c] = r[c] + SF[m - 1][c];
    if (m < N)
      for (int c = 0; c < 4; ++c) r[c] = r[c] + -SF[m][c];
    for (int c = 0; c < 4; ++c) r[c] = 0.0 - r[c];
    if (m == 0)
      for (int c = 0; c < 4; ++c) r[c] = r[c] - BF[0][c];
    if (m == N)
      for (int c = 0; c < 4; ++c) r[c] = r[c] - BF[1][c];
    const double wJq = J * o.wq[m];
    double rl[4];
    for (int c = 0; c < 4; ++c) rl[c] = r[c] / wJq + 0.0;
    st4(a.rhsL + 4 * ((size_t)n * k + m), rl);
    if (a.flags & LF_RHSU_L) st4(a.rhsU + 4 * ((size_t)n * k + m), rl);
    if (a.flags & LF_CFL) {
      const int i = m;
      double li = 0.0;
      for (int j = 0; j < n; ++j) li += (j == i - 1) ? lamR[j] : ((j == i + 1) ? lamR[i] : 0.0);
      if (i == 0 || i == N) {
        const int f = i == 0 ? 0 : 1;
        if (a.flags & LF_LFPROJ) {
          double b0, b1, ut[4];
          Bx(a, k, f, b0, b1);
          ld4(a.uf + 4 * (2 * (size_t)k + f), ut);
          li += find_alpha(U[i], ut, a.POSTOL) * lamB[f] + 0.5 * norm2(b0, b1) * wsf[f];
        } else {
          li += lamB[f];
        }
      }
      scand[e][i] = a.CFL * 0.5 * wJq / li;
    }
  }
  if (!(a.flags & LF_CFL)) return;
  __syncwarp();
  if (live && lane == 0) {
    double dtl = INFINITY;
    for (int i = 0; i < n; ++i) dtl = jmin(dtl, scand[e][i]);
    if (dtl > 0.0)
      atomicMin(&a.dtkey[0], (unsigned long long)__double_as_longlong(dtl));
    else
      atomicOr(a.status, ST_BAD_DT);
  }
}

// initialize_s_modified! (subcell.jl:21-35): the min of phi over all nodes
__global__ void k_line_phimin(LineArgs a) {
  const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= (long long)a.K * a.N1D || done(a) || a.ts[TS_PHI] == 0.0) return;
  double U[4];
  ld4(a.Uq + 4 * g, U);
  atomicMin(a.phikey, encode_key(s_modified4(a.gamma, U)));
}

// the volume two-point terms S_ij fS(u_i, u_j) of flux_differencing_volume!
// (flux_differencing.jl:164-211), one thread per (element, nonzero pair of Srh_db), with
// beta and the logs of each state evaluated as k_line_high evaluates them
__global__ void k_line_pairs(LineArgs a) {
  const LineOps& o = *a.ops;
  const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= (long long)a.K * o.npair || done(a)) return;
  const int k = (int)(g / o.npair), p = (int)(g % o.npair);
  const int n = a.N1D, Nh = n + 2;
  const int i = o.pi[p], j = o.pj[p];
  auto state = [&](int h, double* u) {
    if (h < n)
      ld4(a.Uq + 4 * ((size_t)n * k + h), u);
    else
      ld4(a.uf + 4 * (2 * (size_t)k + (h - n)), u);
  };
  double ui[4], uj[4];
  state(i, ui);
  state(j, uj);
  const double bi = betafun4(a.gamma, ui), bj = betafun4(a.gamma, uj);
  const double Ui[6] = {ui[0], ui[1] / ui[0], ui[2] / ui[0], bi, log(ui[0]), log(bi)};
  const double Uj[6] = {uj[0], uj[1] / uj[0], uj[2] / uj[0], bj, log(uj[0]), log(bj)};
  const double* gg = a.geom + 5 * (size_t)k;
  const double Sr = o.Sh[i + Nh * j], Ss = 0.0;
  const double S0 = gg[1] * Sr + gg[2] * Ss;
  double F[4];
  fS4(a.gamma, Ui, Uj, F);
  double* out = a.sf + (size_t)4 * (kLineMaxPairs * (size_t)k + p);
  for (int c = 0; c < 4; ++c) out[c] = S0 * F[c];
}

// rhs_fluxdiff! (flux_differencing.jl:4-37, 331-361) and the limiter's per-element part:
// Zhang-Shu (zhangshu.jl:4-45) or the subcell factors before symmetrization (subcell.jl:
// Dim1 methods of accumulate_f_bar!, initialize_lower_bound!, initialize_TVD_bounds!,
// subcell_bound_limiter!, enforce_ES_subcell!)
template <int NQ>
__global__ void k_line_high(LineArgs a) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= a.K || done(a)) return;
  constexpr int n = NQ, N = n - 1, Nh = n + 2;
  const int s = a.nstage - 1;
  const LineOps& o = *a.ops;
  const double* g = a.geom + 5 * (size_t)k;
  const double J = g[0];
  const double dt = __longlong_as_double((long long)a.dtkey[1]);  // the limiter's TimeParam dt
  double U[MQ][4], ut[MH][4], QF[MH][4];
  for (int i = 0; i < n; ++i) {
    ld4(a.Uq + 4 * ((size_t)n * k + i), U[i]);
    ld4(U[i], ut[i]);
  }
  for (int f = 0; f < 2; ++f) ld4(a.uf + 4 * (2 * (size_t)k + f), ut[n + f]);
  for (int h = 0; h < Nh; ++h)
    for (int c = 0; c < 4; ++c) QF[h][c] = 0.0;
  // exterior states, interface dissipation coefficients and BCs (:39-151)
  // (the exterior beta and logs of :56-70 enter no flux of this path: the surface flux is
  // LaxFriedrichsOnProjectedVal of the exterior state itself)
  double uP[2][4], LFc[2];
  for (int f = 0; f < 2; ++f) {
    const int fk = 2 * k + f, p = a.nbr[fk], kP = p / 2, iP = p % 2;
    ld4(a.uf + 4 * (size_t)p, uP[f]);
    double b0, b1, c0, c1;
    Bx(a, k, f, b0, b1);
    Bx(a, kP, iP, c0, c1);
    const double nn = norm2(b0, b1), nnP = norm2(c0, c1);
    const double lam = wavespeed4(a.gamma, ut[n + f], b0 / nn, b1 / nn);
    const double lamP = wavespeed4(a.gamma, uP[f], c0 / nnP, c1 / nnP);
    LFc[f] = 0.5 * nn * jmax(lam, lamP);
    const int8_t bc = a.bc[fk];
    if (bc == BC_INFLOW || bc == BC_OUTFLOW) {
      LFc[f] = 0.0;
      if (bc == BC_INFLOW) {
        const double* I = a.Ival + 3 * (size_t)a.bcidx[fk];
        uP[f][0] = I[0], uP[f][1] = I[1], uP[f][2] = 0.0, uP[f][3] = I[2];
      } else {
        ld4(U[f == 0 ? 0 : N], uP[f]);
      }
    }
  }
  // flux_differencing_volume! (:164-211): the pair terms S F of k_line_pairs, accumulated
  // in pair order
  const double* SFk = a.sf + (size_t)4 * kLineMaxPairs * k;
  // each node gathers its pair terms in pair order (the order of the sequential scatter)
#pragma unroll
  for (int h = 0; h < Nh; ++h)
    for (int p = 0; p < o.npair; ++p) {
      const int i = o.pi[p], j = o.pj[p];
      if (i != h && j != h) continue;
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const double SF = SFk[4 * p + c];
        QF[h][c] = QF[h][c] + (i == h ? SF : -SF);
      }
    }
  // flux_differencing_surface! (:223-272)
  double BF[2][4];
  for (int f = 0; f < 2; ++f) {
    double ff[4], fP[4], b0, b1;
    fluxes4(a.gamma, ut[n + f], ff);
    fluxes4(a.gamma, uP[f], fP);
    Bx(a, k, f, b0, b1);
    for (int c = 0; c < 4; ++c) BF[f][c] = b0 * (0.5 * (ff[c] + fP[c])) - LFc[f] * (uP[f][c] - ut[n + f][c]);
    st4(a.BFH + 4 * (2 * (size_t)k + f), BF[f]);
  }
  // assemble_rhs! (:274-361): lift by M \ Vh', or by (1/wq) [I, Vf_new'] when a theta < 1
  const double th0 = a.theta[2 * ((size_t)a.K * s + k)], th1 = a.theta[2 * ((size_t)a.K * s + k) + 1];
  const bool limited = th0 < 1.0 || th1 < 1.0;
  double rH[MQ][4], rL[MQ][4];
  for (int i = 0; i < n; ++i) {
    const double rw = 1 / o.wq[i];
    auto m = [&](int col) -> double {
      if (!limited) return o.MinvVhT[i + n * col];
      if (col < n) return col == i ? rw * 1.0 : 0.0;
      const int f = col - n;
      const double th = f == 0 ? th0 : th1;
      const double low = (i == (f == 0 ? 0 : N)) ? 1.0 : 0.0;
      return rw * (th * o.Vf[f][i] + (1 - th) * low);
    };
    double A[4] = {0, 0, 0, 0}, B[4] = {0, 0, 0, 0};
    for (int j = 0; j < Nh; ++j) {
      const double mm = m(j);
      for (int c = 0; c < 4; ++c) A[c] = A[c] + mm * QF[j][c];
    }
    for (int f = 0; f < 2; ++f) {
      const double mm = m(n + f);
      for (int c = 0; c < 4; ++c) B[c] = B[c] + mm * BF[f][c];
    }
    for (int c = 0; c < 4; ++c) rH[i][c] = -(A[c] + B[c]) / J;
    st4(a.rhsH + 4 * ((size_t)n * k + i), rH[i]);
    ld4(a.rhsL + 4 * ((size_t)n * k + i), rL[i]);
    if (a.flags & LF_RHSU_H) st4(a.rhsU + 4 * ((size_t)n * k + i), rH[i]);
  }
  if (!(a.flags & (LF_ZS | LF_SUBCELL))) return;
  double blend, epsk;
  smoothness(a, U, blend, epsk);
  const double zeta = a.zeta;
  if (a.flags & LF_ZS) {  // zhang_shu_bound_limiter! (zhangshu.jl:35-45)
    double l = 1.0;
    for (int i = 0; i < n; ++i) {
      double uL[4], P[4];
      for (int c = 0; c < 4; ++c) {
        uL[c] = U[i][c] + dt * rL[i][c];
        P[c] = dt * (rH[i][c] - rL[i][c]);
      }
      const double li = jmin(1.0, bound_rho_rhoe(uL, P, zeta * uL[0], zeta * rhoe4(uL), INFINITY, INFINITY, a.ZEROTOL));
      l = jmin(l, li);
    }
    a.Lelem[(size_t)a.K * s + k] = l;
    l = jmin(l, blend);
    for (int i = 0; i < n; ++i) {
      double r[4];
      for (int c = 0; c < 4; ++c) r[c] = (1 - l) * rL[i][c] + l * rH[i][c];
      st4(a.rhsU + 4 * ((size_t)n * k + i), r);
    }
    return;
  }
  // the two-point stencil of node q (low_order_stencil(::Dim1), limiter_utils.jl:184-220)
  auto stencil = [&](int q, int* kk, int* qq) {
    for (int t = 0; t < 2; ++t) {
      const int qn = q + (t == 0 ? -1 : 1);
      if (qn >= 0 && qn <= N) {
        kk[t] = k;
        qq[t] = qn;
      } else {
        const int p = a.nbr[2 * k + (q == 0 ? 0 : 1)];
        kk[t] = p / 2;
        qq[t] = (p % 2 == 0) ? 0 : N;
      }
    }
  };
  double Lphi[MQ], Lrho[MQ], Urho[MQ];
  double uL[MQ][4];
  const double phimin = decode_key(*a.phikey);
  for (int q = 0; q < n; ++q) {
    for (int c = 0; c < 4; ++c) uL[q][c] = U[q][c] + dt * rL[q][c];
    int kk[2], qq[2];
    stencil(q, kk, qq);
    Lphi[q] = 0.0;
    if (a.flags & LF_MINENT) {  // initialize_lower_bound!(::Dim1) (subcell.jl:37-51)
      double lb = s_modified4(a.gamma, U[q]);
      for (int t = 0; t < 2; ++t) {
        double Un[4];
        ld4(a.Uq + 4 * ((size_t)n * kk[t] + qq[t]), Un);
        lb = jmin(lb, s_modified4(a.gamma, Un));
      }
      Lphi[q] = epsk * lb + (1 - epsk) * phimin;
    }
    Lrho[q] = zeta * uL[q][0];
    Urho[q] = INFINITY;
    if (a.flags & LF_TVD) {  // initialize_TVD_bounds!(::Dim1) (:86-110)
      double lb = U[q][0] + dt * rL[q][0], ub = lb;
      for (int t = 0; t < 2; ++t) {
        const size_t m = (size_t)n * kk[t] + qq[t];
        const double v = a.Uq[4 * m] + dt * a.rhsL[4 * m];
        lb = jmin(lb, v);
        ub = jmax(ub, v);
      }
      Lrho[q] = lb;
      Urho[q] = ub;
    }
  }
  // accumulate_f_bar!(::Dim1) (:144-160)
  double fH[MQ + 1][4], fL[MQ + 1][4];
  ld4(BF[0], fH[0]);
  ld4(a.BFL + 4 * (2 * (size_t)k), fL[0]);
  for (int i = 1; i <= n; ++i) {
    const double wJ = J * o.wq[i - 1];
    for (int c = 0; c < 4; ++c) {
      fH[i][c] = fH[i - 1][c] + wJ * rH[i - 1][c];
      fL[i][c] = fL[i - 1][c] + wJ * rL[i - 1][c];
    }
  }
  // subcell_bound_limiter!(::Dim1) (:208-246)
  double L[MS];
  for (int i = 0; i < 2 * n; ++i) L[i] = 1.0;
  auto eval = [&](int q, int i, double sgn) {
    const double wJ = o.wq[q] * J;
    double P[4];
    for (int c = 0; c < 4; ++c) P[c] = sgn * 2.0 * dt * (fH[i][c] - fL[i][c]) / wJ;
    const double Lrhoe = zeta * rhoe4(uL[q]);
    const double lpos = bound_rho_rhoe(uL[q], P, Lrho[q], Lrhoe, Urho[q], INFINITY, a.ZEROTOL);
    if (!(a.flags & LF_MINENT)) return lpos;
    // limiting_param_bound_phi (limiter_utils.jl:43-50) by bisection on [0, lpos]
    const double thr = Lphi[q] - a.POSTOL;
    auto okp = [&](double l) {
      double W[4];
      for (int c = 0; c < 4; ++c) W[c] = uL[q][c] + l * P[c];
      return s_modified4(a.gamma, W) >= thr;
    };
    double x_valid = 0.0, x_invalid = lpos;
    if (okp(x_invalid)) return x_invalid;
    for (int iter = 0; iter <= 20; ++iter) {
      const double x_new = 0.5 * (x_valid + x_invalid);
      if (okp(x_new))
        x_valid = x_new;
      else
        x_invalid = x_new;
    }
    return x_valid;
  };
  for (int i = 0; i < n; ++i) L[i] = jmin(L[i], eval(i, i, -1.0));
  for (int i = 1; i <= n; ++i) L[i] = jmin(L[i], eval(i - 1, i, 1.0));
  for (int i = 0; i < 2 * n; ++i) L[i] = jmin(L[i], blend);
  if (a.flags & LF_CELL) {  // Dim1 methods of subcell.jl:468-505, 567-628, rhs_es :746-753
    double v[MQ][4];
    for (int i = 0; i < n; ++i) v_ufun4(a.gamma, U[i], v[i]);
    double sB = 0.0;
    for (int f = 0; f < 2; ++f) {
      double b0, b1;
      Bx(a, k, f, b0, b1);
      const double psi = (a.gamma - 1.0) * U[f == 0 ? 0 : N][1];
      sB = sB + b0 * psi;
    }
    double d[MQ], sx = 0.0;
    for (int si = 1; si <= N; ++si) {
      double dvdf = 0.0, dvfl = 0.0;
      double t1[4], t2[4];
      for (int c = 0; c < 4; ++c) {
        const double dv = v[si - 1][c] - v[si][c];
        t1[c] = dv * (fH[si][c] - fL[si][c]);
        t2[c] = dv * fL[si][c];
      }
      dvdf = ((t1[0] + t1[1]) + t1[2]) + t1[3];
      dvfl = ((t2[0] + t2[1]) + t2[2]) + t2[3];
      d[si - 1] = dvdf;
      sx += dvfl;
    }
    double sum = 0.0;
    for (int si = 1; si <= N; ++si) sum += L[si] * d[si - 1];
    double rhs = sB - sx;
    if (a.flags & LF_RELAXED) rhs = (1 - a.beta * epsk) * rhs;
    const double tol = jmax(0.0, sx - sB);
    if (sum - rhs > tol) {
      // indices 1..N by dvdf descending (sort!(..., rev=true) on (value, index) tuples)
      int order[MQ];
      for (int i = 0; i < N; ++i) order[i] = i + 1;
      for (int i = 1; i < N; ++i)
        for (int j = i; j > 0; --j) {
          const int x = order[j - 1], y = order[j];
          const bool y_first = jisless(d[x - 1], d[y - 1]) || (!jisless(d[y - 1], d[x - 1]) && x < y);
          if (!y_first) break;
          order[j - 1] = y;
          order[j] = x;
        }
      int curr = 1;
      double lhs = sum;
      while (lhs > rhs + tol && curr <= n - 1) {
        const int idx = order[curr - 1];
        if (d[idx - 1] < a.ZEROTOL) break;
        lhs = lhs - L[idx] * d[idx - 1];
        curr += 1;
      }
      for (int i = 1; i <= curr - 1; ++i) {
        const int idx = order[i - 1];
        const double l_new = (i == curr - 1) ? jmax((rhs + tol - lhs) / d[idx - 1], 0.0) : 0.0;
        L[idx] = jmin(L[idx], l_new);
      }
    }
  }
  double* Lr = a.Lraw + (size_t)2 * n * k;
  for (int i = 0; i < 2 * n; ++i) Lr[i] = L[i];
  double* fb = a.fbar + (size_t)8 * (n + 1) * k;
  for (int i = 0; i <= n; ++i) {
    st4(fb + 4 * i, fH[i]);
    st4(fb + 4 * (n + 1 + i), fL[i]);
  }
}

// k_line_high with a team of kTeam lanes per element (kTeamE elements per one-warp block),
// for solves too small to fill the GPU one thread per element: there each element's work is
// one long dependent chain, so its independent parts — the rows of the gather and the lift,
// the two faces, the nodes' bounds, the eight prefix-sum columns and the 2n bound
// evaluations — run on separate lanes. Every value is formed by the same expression, in the
// same order, as in k_line_high (this unit is compiled without FMA contraction), so both
// kernels give the same bits; the sequential parts (the smoothness factor, the cell-entropy
// sums and greedy) run on every lane or on the team's first lane.
template <int NQ>
__global__ void k_line_high_team(LineArgs a) {
  constexpr int n = NQ, N = n - 1, Nh = n + 2, E = kTeamE;
  static_assert(2 * n <= kTeam && Nh <= kTeam, "one lane per evaluation and per gather row");
  const int lane = threadIdx.x % kTeam, e = threadIdx.x / kTeam;
  const int k = blockIdx.x * E + e;
  if (done(a)) return;  // the same for the whole grid
  const bool live = k < a.K;
  const int s = a.nstage - 1;
  const LineOps& o = *a.ops;
  __shared__ double sU[E][n][4], sut[E][Nh][4], sQF[E][Nh][4], suP[E][2][4], sLFc[E][2], sBF[E][2][4];
  __shared__ double srH[E][n][4], srL[E][n][4], sli[E][n], suL[E][n][4], sLphi[E][n], sLrho[E][n], sUrho[E][n];
  __shared__ double sfH[E][n + 1][4], sfL[E][n + 1][4], sev[E][2 * n], sL[E][2 * n], sv[E][n][4];
  double(*U)[4] = sU[e];
  double(*ut)[4] = sut[e];
  double(*QF)[4] = sQF[e];
  double(*uP)[4] = suP[e];
  double* LFc = sLFc[e];
  double(*BF)[4] = sBF[e];
  double(*rH)[4] = srH[e];
  double(*rL)[4] = srL[e];
  const double J = live ? a.geom[5 * (size_t)k] : 1.0;
  const double dt = __longlong_as_double((long long)a.dtkey[1]);  // the limiter's TimeParam dt
  if (live) {
    if (lane < n) {
      ld4(a.Uq + 4 * ((size_t)n * k + lane), U[lane]);
      ld4(U[lane], ut[lane]);
    } else if (lane < Nh) {
      ld4(a.uf + 4 * (2 * (size_t)k + (lane - n)), ut[lane]);
    }
    if (lane < Nh)
      for (int c = 0; c < 4; ++c) QF[lane][c] = 0.0;
  }
  __syncwarp();
  // exterior states, interface dissipation coefficients and BCs (:39-151), one lane per face
  if (live && lane < 2) {
    const int f = lane;
    const int fk = 2 * k + f, p = a.nbr[fk], kP = p / 2, iP = p % 2;
    ld4(a.uf + 4 * (size_t)p, uP[f]);
    double b0, b1, c0, c1;
    Bx(a, k, f, b0, b1);
    Bx(a, kP, iP, c0, c1);
    const double nn = norm2(b0, b1), nnP = norm2(c0, c1);
    const double lam = wavespeed4(a.gamma, ut[n + f], b0 / nn, b1 / nn);
    const double lamP = wavespeed4(a.gamma, uP[f], c0 / nnP, c1 / nnP);
    LFc[f] = 0.5 * nn * jmax(lam, lamP);
    const int8_t bc = a.bc[fk];
    if (bc == BC_INFLOW || bc == BC_OUTFLOW) {
      LFc[f] = 0.0;
      if (bc == BC_INFLOW) {
        const double* I = a.Ival + 3 * (size_t)a.bcidx[fk];
        uP[f][0] = I[0], uP[f][1] = I[1], uP[f][2] = 0.0, uP[f][3] = I[2];
      } else {
        ld4(U[f == 0 ? 0 : N], uP[f]);
      }
    }
  }
  // flux_differencing_volume! (:164-211): one lane per row h gathers its pair terms in
  // pair order
  if (live && lane < Nh) {
    const int h = lane;
    const double* SFk = a.sf + (size_t)4 * kLineMaxPairs * k;
    for (int p = 0; p < o.npair; ++p) {
      const int i = o.pi[p], j = o.pj[p];
      if (i != h && j != h) continue;
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const double SF = SFk[4 * p + c];
        QF[h][c] = QF[h][c] + (i == h ? SF : -SF);
      }
    }
  }
  __syncwarp();
  // flux_differencing_surface! (:223-272), one lane per face
  if (live && lane < 2) {
    const int f = lane;
    double ff[4], fP[4], b0, b1;
    fluxes4(a.gamma, ut[n + f], ff);
    fluxes4(a.gamma, uP[f], fP);
    Bx(a, k, f, b0, b1);
    for (int c = 0; c < 4; ++c) BF[f][c] = b0 * (0.5 * (ff[c] + fP[c])) - LFc[f] * (uP[f][c] - ut[n + f][c]);
    st4(a.BFH + 4 * (2 * (size_t)k + f), BF[f]);
  }
  __syncwarp();
  // assemble_rhs! (:274-361), one lane per row i
  const double th0 = live ? a.theta[2 * ((size_t)a.K * s + k)] : 1.0;
  const double th1 = live ? a.theta[2 * ((size_t)a.K * s + k) + 1] : 1.0;
  const bool limited = th0 < 1.0 || th1 < 1.0;
  if (live && lane < n) {
    const int i = lane;
    const double rw = 1 / o.wq[i];
    auto m = [&](int col) -> double {
      if (!limited) return o.MinvVhT[i + n * col];
      if (col < n) return col == i ? rw * 1.0 : 0.0;
      const int f = col - n;
      const double th = f == 0 ? th0 : th1;
      const double low = (i == (f == 0 ? 0 : N)) ? 1.0 : 0.0;
      return rw * (th * o.Vf[f][i] + (1 - th) * low);
    };
    double A[4] = {0, 0, 0, 0}, B[4] = {0, 0, 0, 0};
    for (int j = 0; j < Nh; ++j) {
      const double mm = m(j);
      for (int c = 0; c < 4; ++c) A[c] = A[c] + mm * QF[j][c];
    }
    for (int f = 0; f < 2; ++f) {
      const double mm = m(n + f);
      for (int c = 0; c < 4; ++c) B[c] = B[c] + mm * BF[f][c];
    }
    for (int c = 0; c < 4; ++c) rH[i][c] = -(A[c] + B[c]) / J;
    st4(a.rhsH + 4 * ((size_t)n * k + i), rH[i]);
    ld4(a.rhsL + 4 * ((size_t)n * k + i), rL[i]);
    if (a.flags & LF_RHSU_H) st4(a.rhsU + 4 * ((size_t)n * k + i), rH[i]);
  }
  if (!(a.flags & (LF_ZS | LF_SUBCELL))) return;
  __syncwarp();
  double blend = 1.0, epsk = 0.0;
  if (live) smoothness(a, U, blend, epsk);  // on every lane, from the same shared state
  const double zeta = a.zeta;
  if (a.flags & LF_ZS) {  // zhang_shu_bound_limiter! (zhangshu.jl:35-45)
    if (live && lane < n) {
      const int i = lane;
      double uL[4], P[4];
      for (int c = 0; c < 4; ++c) {
        uL[c] = U[i][c] + dt * rL[i][c];
        P[c] = dt * (rH[i][c] - rL[i][c]);
      }
      sli[e][i] = jmin(1.0, bound_rho_rhoe(uL, P, zeta * uL[0], zeta * rhoe4(uL), INFINITY, INFINITY, a.ZEROTOL));
    }
    __syncwarp();
    if (live && lane < n) {
      double l = 1.0;
      for (int i = 0; i < n; ++i) l = jmin(l, sli[e][i]);
      if (lane == 0) a.Lelem[(size_t)a.K * s + k] = l;
      l = jmin(l, blend);
      const int i = lane;
      double r[4];
      for (int c = 0; c < 4; ++c) r[c] = (1 - l) * rL[i][c] + l * rH[i][c];
      st4(a.rhsU + 4 * ((size_t)n * k + i), r);
    }
    return;
  }
  double(*uL)[4] = suL[e];
  double *Lphi = sLphi[e], *Lrho = sLrho[e], *Urho = sUrho[e];
  // node bounds, one lane per node
  if (live && lane < n) {
    const int q = lane;
    const double phimin = decode_key(*a.phikey);
    for (int c = 0; c < 4; ++c) uL[q][c] = U[q][c] + dt * rL[q][c];
    // the two-point stencil of node q (low_order_stencil(::Dim1), limiter_utils.jl:184-220)
    int kk[2], qq[2];
    for (int t = 0; t < 2; ++t) {
      const int qn = q + (t == 0 ? -1 : 1);
      if (qn >= 0 && qn <= N) {
        kk[t] = k;
        qq[t] = qn;
      } else {
        const int p = a.nbr[2 * k + (q == 0 ? 0 : 1)];
        kk[t] = p / 2;
        qq[t] = (p % 2 == 0) ? 0 : N;
      }
    }
    Lphi[q] = 0.0;
    if (a.flags & LF_MINENT) {  // initialize_lower_bound!(::Dim1) (subcell.jl:37-51)
      double lb = s_modified4(a.gamma, U[q]);
      for (int t = 0; t < 2; ++t) {
        double Un[4];
        ld4(a.Uq + 4 * ((size_t)n * kk[t] + qq[t]), Un);
        lb = jmin(lb, s_modified4(a.gamma, Un));
      }
      Lphi[q] = epsk * lb + (1 - epsk) * phimin;
    }
    Lrho[q] = zeta * uL[q][0];
    Urho[q] = INFINITY;
    if (a.flags & LF_TVD) {  // initialize_TVD_bounds!(::Dim1) (:86-110)
      double lb = U[q][0] + dt * rL[q][0], ub = lb;
      for (int t = 0; t < 2; ++t) {
        const size_t m = (size_t)n * kk[t] + qq[t];
        const double v = a.Uq[4 * m] + dt * a.rhsL[4 * m];
        lb = jmin(lb, v);
        ub = jmax(ub, v);
      }
      Lrho[q] = lb;
      Urho[q] = ub;
    }
  }
  // accumulate_f_bar!(::Dim1) (:144-160), one lane per (H or L, component)
  double(*fH)[4] = sfH[e];
  double(*fL)[4] = sfL[e];
  if (live && lane < 8) {
    const int c = lane % 4;
    const bool hi = lane < 4;
    double(*fb)[4] = hi ? fH : fL;
    double(*r)[4] = hi ? rH : rL;
    fb[0][c] = hi ? BF[0][c] : a.BFL[4 * (2 * (size_t)k) + c];
    for (int i = 1; i <= n; ++i) {
      const double wJ = J * o.wq[i - 1];
      fb[i][c] = fb[i - 1][c] + wJ * r[i - 1][c];
    }
  }
  __syncwarp();
  // subcell_bound_limiter!(::Dim1) (:208-246): the 2n evaluations, one lane each; lane i < n
  // limits face i from node i (sign -1), lane n + i - 1 face i from node i - 1 (sign +1)
  double* ev = sev[e];
  if (live && lane < 2 * n) {
    const int q = lane < n ? lane : lane - n;
    const int i = lane < n ? lane : lane - n + 1;
    const double sgn = lane < n ? -1.0 : 1.0;
    const double wJ = o.wq[q] * J;
    double P[4];
    for (int c = 0; c < 4; ++c) P[c] = sgn * 2.0 * dt * (fH[i][c] - fL[i][c]) / wJ;
    const double Lrhoe = zeta * rhoe4(uL[q]);
    double l = bound_rho_rhoe(uL[q], P, Lrho[q], Lrhoe, Urho[q], INFINITY, a.ZEROTOL);
    if (a.flags & LF_MINENT) {
      // limiting_param_bound_phi (limiter_utils.jl:43-50) by bisection on [0, lpos]
      const double thr = Lphi[q] - a.POSTOL;
      auto okp = [&](double lv) {
        double W[4];
        for (int c = 0; c < 4; ++c) W[c] = uL[q][c] + lv * P[c];
        return s_modified4(a.gamma, W) >= thr;
      };
      double x_valid = 0.0, x_invalid = l;
      if (!okp(x_invalid)) {
        for (int iter = 0; iter <= 20; ++iter) {
          const double x_new = 0.5 * (x_valid + x_invalid);
          if (okp(x_new))
            x_valid = x_new;
          else
            x_invalid = x_new;
        }
        l = x_valid;
      }
    }
    ev[lane] = l;
  }
  __syncwarp();
  double* L = sL[e];
  if (live && lane < 2 * n) {
    const int i = lane;
    double Li = 1.0;
    if (i < n) Li = jmin(Li, ev[i]);
    if (i >= 1 && i <= n) Li = jmin(Li, ev[n + i - 1]);
    L[i] = jmin(Li, blend);
  }
  __syncwarp();
  if (a.flags & LF_CELL) {  // Dim1 methods of subcell.jl:468-505, 567-628, rhs_es :746-753
    double(*v)[4] = sv[e];
    if (live && lane < n) v_ufun4(a.gamma, U[lane], v[lane]);
    __syncwarp();
    if (live && lane == 0) {
      double sB = 0.0;
      for (int f = 0; f < 2; ++f) {
        double b0, b1;
        Bx(a, k, f, b0, b1);
        const double psi = (a.gamma - 1.0) * U[f == 0 ? 0 : N][1];
        sB = sB + b0 * psi;
      }
      double d[MQ], sx = 0.0;
      for (int si = 1; si <= N; ++si) {
        double dvdf = 0.0, dvfl = 0.0;
        double t1[4], t2[4];
        for (int c = 0; c < 4; ++c) {
          const double dv = v[si - 1][c] - v[si][c];
          t1[c] = dv * (fH[si][c] - fL[si][c]);
          t2[c] = dv * fL[si][c];
        }
        dvdf = ((t1[0] + t1[1]) + t1[2]) + t1[3];
        dvfl = ((t2[0] + t2[1]) + t2[2]) + t2[3];
        d[si - 1] = dvdf;
        sx += dvfl;
      }
      double sum = 0.0;
      for (int si = 1; si <= N; ++si) sum += L[si] * d[si - 1];
      double rhs = sB - sx;
      if (a.flags & LF_RELAXED) rhs = (1 - a.beta * epsk) * rhs;
      const double tol = jmax(0.0, sx - sB);
      if (sum - rhs > tol) {
        // indices 1..N by dvdf descending (sort!(..., rev=true) on (value, index) tuples)
        int order[MQ];
        for (int i = 0; i < N; ++i) order[i] = i + 1;
        for (int i = 1; i < N; ++i)
          for (int j = i; j > 0; --j) {
            const int x = order[j - 1], y = order[j];
            const bool y_first = jisless(d[x - 1], d[y - 1]) || (!jisless(d[y - 1], d[x - 1]) && x < y);
            if (!y_first) break;
            order[j - 1] = y;
            order[j] = x;
          }
        int curr = 1;
        double lhs = sum;
        while (lhs > rhs + tol && curr <= n - 1) {
          const int idx = order[curr - 1];
          if (d[idx - 1] < a.ZEROTOL) break;
          lhs = lhs - L[idx] * d[idx - 1];
          curr += 1;
        }
        for (int i = 1; i <= curr - 1; ++i) {
          const int idx = order[i - 1];
          const double l_new = (i == curr - 1) ? jmax((rhs + tol - lhs) / d[idx - 1], 0.0) : 0.0;
          L[idx] = jmin(L[idx], l_new);
        }
      }
    }
  }
  __syncwarp();
  if (live && lane < 2 * n) a.Lraw[(size_t)2 * n * k + lane] = L[lane];
  if (live && lane <= n) {
    double* fb = a.fbar + (size_t)8 * (n + 1) * k;
    st4(fb + 4 * lane, fH[lane]);
    st4(fb + 4 * (n + 1 + lane), fL[lane]);
  }
}

// symmetrize_limiting_parameters!(::Dim1) (subcell.jl:405-415) across mapP,
// accumulate_f_bar_limited!(::Dim1) (:826-839), apply_subcell_limiter!(::Dim1) (:878-892);
// then the SSP-RK3 stage update (SSPRK33.jl:125-139) and the positivity record
template <int NQ>
__global__ void k_line_update(LineArgs a) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= a.K || done(a)) return;
  constexpr int n = NQ;
  const int s = a.nstage - 1;
  const LineOps& o = *a.ops;
  const double J = a.geom[5 * (size_t)k];
  double* rU = a.rhsU + 4 * (size_t)n * k;
  if (a.flags & LF_SUBCELL) {
    const double* Lr = a.Lraw + (size_t)2 * n * k;
    double L[MS];
    for (int i = 0; i < 2 * n; ++i) L[i] = Lr[i];
    for (int f = 0; f < 2; ++f) {
      const int p = a.nbr[2 * k + f], kP = p / 2, iP = p % 2;
      const int si = f == 0 ? 0 : n, siP = iP == 0 ? 0 : n;
      L[si] = jmin(Lr[si], a.Lraw[(size_t)2 * n * kP + siP]);
    }
    double* Lo = a.Lloc + (size_t)2 * n * ((size_t)a.K * s + k);
    for (int i = 0; i < 2 * n; ++i) Lo[i] = L[i];
    const double* fb = a.fbar + (size_t)8 * (n + 1) * k;
    double flim[MQ + 1][4];
    for (int i = 0; i <= n; ++i)
      for (int c = 0; c < 4; ++c) flim[i][c] = L[i] * fb[4 * i + c] + (1.0 - L[i]) * fb[4 * (n + 1 + i) + c];
    for (int i = 0; i < n; ++i) {
      const double wJ = o.wq[i] * J;
      for (int c = 0; c < 4; ++c) rU[4 * i + c] = (flim[i + 1][c] - flim[i][c]) / wJ;
    }
  }
  if (!(a.flags & LF_UPDATE)) return;
  const double dt = __longlong_as_double((long long)a.dtkey[0]);  // the step's dt
  double rmin = INFINITY, emin = INFINITY;
  int bad = 0;
  for (int i = 0; i < n; ++i) {
    double* u = a.Uq + 4 * ((size_t)n * k + i);
    double* w = a.resW + 4 * ((size_t)n * k + i);
    for (int c = 0; c < 4; ++c) {
      if (a.nstage == 1) {
        w[c] = u[c];
        u[c] = w[c] + dt * rU[4 * i + c];
      } else {
        const double z = u[c] + dt * rU[4 * i + c];
        u[c] = a.nstage == 2 ? 3.0 / 4.0 * w[c] + 1.0 / 4.0 * z : 1.0 / 3.0 * w[c] + 2.0 / 3.0 * z;
      }
    }
    const double re = rhoe4(u);
    if (isnan(u[0]) || isnan(re)) bad |= ST_NAN;
    if (!(u[0] > 0.0) || !(re > 0.0)) bad |= ST_NOT_POSITIVE;
    rmin = fmin(rmin, u[0]);
    emin = fmin(emin, re);
  }
  if (bad) atomicOr(a.status, bad);
  atomicMin(&a.minrec[2 * s], encode_key(rmin));
  atomicMin(&a.minrec[2 * s + 1], encode_key(emin));
}

// k_line_update with a team of kTeam lanes per element: the symmetrized factors, the limited
// subcell fluxes and the nodes' rhsU and stage update on separate lanes, each value formed as
// in k_line_update (same bits); the element's minima are taken in node order on the team's
// first lane.
template <int NQ>
__global__ void k_line_update_team(LineArgs a) {
  constexpr int n = NQ, E = kTeamE;
  static_assert(2 * n <= kTeam, "one lane per factor");
  const int lane = threadIdx.x % kTeam, e = threadIdx.x / kTeam;
  const int k = blockIdx.x * E + e;
  if (done(a)) return;  // the same for the whole grid
  const bool live = k < a.K;
  const int s = a.nstage - 1;
  const LineOps& o = *a.ops;
  __shared__ double sL[E][2 * n], sflim[E][n + 1][4], smin[E][n][2];
  const double J = live ? a.geom[5 * (size_t)k] : 1.0;
  double* rU = a.rhsU + 4 * (size_t)n * (live ? k : 0);
  double ru[4];
  if (a.flags & LF_SUBCELL) {
    double* L = sL[e];
    if (live && lane < 2 * n) {
      const double* Lr = a.Lraw + (size_t)2 * n * k;
      double Li = Lr[lane];
      for (int f = 0; f < 2; ++f) {
        const int si = f == 0 ? 0 : n;
        if (lane != si) continue;
        const int p = a.nbr[2 * k + f], kP = p / 2, iP = p % 2;
        const int siP = iP == 0 ? 0 : n;
        Li = jmin(Lr[si], a.Lraw[(size_t)2 * n * kP + siP]);
      }
      L[lane] = Li;
      a.Lloc[(size_t)2 * n * ((size_t)a.K * s + k) + lane] = Li;
    }
    __syncwarp();
    double(*flim)[4] = sflim[e];
    if (live && lane <= n) {
      const int i = lane;
      const double* fb = a.fbar + (size_t)8 * (n + 1) * k;
      for (int c = 0; c < 4; ++c) flim[i][c] = L[i] * fb[4 * i + c] + (1.0 - L[i]) * fb[4 * (n + 1 + i) + c];
    }
    __syncwarp();
    if (live && lane < n) {
      const int i = lane;
      const double wJ = o.wq[i] * J;
      for (int c = 0; c < 4; ++c) {
        ru[c] = (flim[i + 1][c] - flim[i][c]) / wJ;
        rU[4 * i + c] = ru[c];
      }
    }
  } else if (live && lane < n) {
    for (int c = 0; c < 4; ++c) ru[c] = rU[4 * lane + c];
  }
  if (!(a.flags & LF_UPDATE)) return;
  const double dt = __longlong_as_double((long long)a.dtkey[0]);  // the step's dt
  if (live && lane < n) {
    const int i = lane;
    double* u = a.Uq + 4 * ((size_t)n * k + i);
    double* w = a.resW + 4 * ((size_t)n * k + i);
    for (int c = 0; c < 4; ++c) {
      if (a.nstage == 1) {
        w[c] = u[c];
        u[c] = w[c] + dt * ru[c];
      } else {
        const double z = u[c] + dt * ru[c];
        u[c] = a.nstage == 2 ? 3.0 / 4.0 * w[c] + 1.0 / 4.0 * z : 1.0 / 3.0 * w[c] + 2.0 / 3.0 * z;
      }
    }
    const double re = rhoe4(u);
    int bad = 0;
    if (isnan(u[0]) || isnan(re)) bad |= ST_NAN;
    if (!(u[0] > 0.0) || !(re > 0.0)) bad |= ST_NOT_POSITIVE;
    if (bad) atomicOr(a.status, bad);
    smin[e][i][0] = u[0];
    smin[e][i][1] = re;
  }
  __syncwarp();
  if (live && lane == 0) {
    double rmin = INFINITY, emin = INFINITY;
    for (int i = 0; i < n; ++i) {
      rmin = fmin(rmin, smin[e][i][0]);
      emin = fmin(emin, smin[e][i][1]);
    }
    atomicMin(&a.minrec[2 * s], encode_key(rmin));
    atomicMin(&a.minrec[2 * s + 1], encode_key(emin));
  }
}

template <typename T>
cudaError_t dalloc(LineSolve* L, T** p, size_t count) {
  void* q = nullptr;
  const size_t bytes = sizeof(T) * (count > 0 ? count : 1);
  cudaError_t e = cudaMalloc(&q, bytes);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(q, 0, bytes, L->stream);
  if (e != cudaSuccess) return e;
  L->allocs.push_back(q);
  *p = (T*)q;
  return cudaSuccess;
}

bool is_one_of(int b, std::initializer_list<int> l) {
  for (int x : l)
    if (b == x) return true;
  return false;
}

int line_flags(const LineSolve* L, int nstage, bool update) {
  const p2de_param& p = L->prm;
  int f = 0;
  switch (p.rhs_type) {
    case P2DE_RHS_LOW_ORDER_POSITIVITY: f |= LF_LOW | LF_RHSU_L; break;
    case P2DE_RHS_ENTROPY_STABLE: f |= LF_HIGH | LF_RHSU_H; break;
    default: f |= LF_LOW | LF_HIGH | (p.rhs_limiter == P2DE_LIMITER_ZHANG_SHU ? LF_ZS : LF_SUBCELL); break;
  }
  if ((f & LF_LOW) && nstage == 1) f |= LF_CFL;
  if (p.low_order_surface_flux == P2DE_FLUX_LAX_FRIEDRICHS_ON_PROJECTED_VAL) f |= LF_LFPROJ;
  if (p.approximation_basis == P2DE_BASIS_GAUSS && p.entropyproj_limiter == P2DE_ENTROPYPROJ_NODEWISE_SCALED_EXTRAPOLATION)
    f |= LF_NSE;
  if ((f & (LF_ZS | LF_SUBCELL)) && p.shock_capture == 1) f |= LF_SHOCK;
  if (f & LF_SUBCELL) {
    const int b = p.bound_type;
    if (is_one_of(b, {P2DE_BOUND_TVD, P2DE_BOUND_TVD_AND_CELL_ENTROPY, P2DE_BOUND_TVD_AND_MIN_ENTROPY,
                      P2DE_BOUND_TVD_AND_RELAXED_MIN_ENTROPY, P2DE_BOUND_TVD_AND_RELAXED_CELL_ENTROPY}))
      f |= LF_TVD;
    if (is_one_of(b, {P2DE_BOUND_POSITIVITY_AND_MIN_ENTROPY, P2DE_BOUND_POSITIVITY_AND_RELAXED_MIN_ENTROPY,
                      P2DE_BOUND_TVD_AND_MIN_ENTROPY, P2DE_BOUND_TVD_AND_RELAXED_MIN_ENTROPY}))
      f |= LF_MINENT;
    if (is_one_of(b, {P2DE_BOUND_POSITIVITY_AND_RELAXED_MIN_ENTROPY, P2DE_BOUND_TVD_AND_RELAXED_MIN_ENTROPY,
                      P2DE_BOUND_POSITIVITY_AND_RELAXED_CELL_ENTROPY, P2DE_BOUND_TVD_AND_RELAXED_CELL_ENTROPY}))
      f |= LF_RELAXED;
    if (is_one_of(b, {P2DE_BOUND_POSITIVITY_AND_CELL_ENTROPY, P2DE_BOUND_TVD_AND_CELL_ENTROPY,
                      P2DE_BOUND_POSITIVITY_AND_RELAXED_CELL_ENTROPY, P2DE_BOUND_TVD_AND_RELAXED_CELL_ENTROPY}))
      f |= LF_CELL;
  }
  if (update) f |= LF_UPDATE;
  return f;
}

LineArgs args_of(const LineSolve* L, int nstage, int flags) {
  const p2de_param& p = L->prm;
  LineArgs a{};
  a.K = L->K;
  a.N1D = L->N1D;
  a.nstage = nstage;
  a.flags = flags;
  a.ops = L->ops;
  a.Uq = L->Uq;
  a.resW = L->resW;
  a.rhsL = L->rhsL;
  a.rhsH = L->rhsH;
  a.rhsU = L->rhsU;
  a.BFL = L->BFL;
  a.BFH = L->BFH;
  a.uf = L->uf;
  a.theta = L->theta;
  a.Lloc = L->Lloc;
  a.Lraw = L->Lraw;
  a.fbar = L->fbar;
  a.Lelem = L->Lelem;
  a.sf = L->sf;
  a.geom = L->geom;
  a.Ival = L->Ival;
  a.phikey = reinterpret_cast<long long*>(L->phimin);
  a.nbr = L->nbr;
  a.bcidx = L->bcidx;
  a.bc = L->bc;
  a.dtkey = L->dtkey;
  a.minrec = L->minrec;
  a.status = L->status;
  a.ts = L->ts;
  a.T = p.T;
  a.dt0 = p.dt0;
  a.t0 = p.t0;
  a.gamma = p.gamma;
  a.POSTOL = p.POSTOL;
  a.ZEROTOL = p.ZEROTOL;
  a.zeta = p.zeta;
  a.eta = p.eta;
  a.CFL = p.CFL;
  a.beta = p.bound_beta;
  // HennemannShockCapture (shock_capture.jl:118-137): threshold and sigmoid sharpness
  const int N = L->N1D - 1;
  a.sc_TN = p.shock_capture_a * std::pow(10.0, -p.shock_capture_c * std::pow((double)(N + 1), 0.25));
  a.sc_sfac = std::log((1 - 0.0001) / 0.0001);
  a.s0 = std::log(1.0 / ((double)N * N * N * N)) / std::log(10.0);
  return a;
}

double host_jmin(double x, double y) {
  if (std::isnan(x) || std::isnan(y)) return NAN;
  if (x == y) return std::signbit(x) ? x : y;
  return x < y ? x : y;
}

// kern<N1D> for the solve's degree
#define LINE_LAUNCH(kern, grid, args)                                            \
  switch (L->N1D) {                                                              \
    case 2: kern<2><<<(grid), kThreads, 0, L->stream>>>(args); break;            \
    case 3: kern<3><<<(grid), kThreads, 0, L->stream>>>(args); break;            \
    case 4: kern<4><<<(grid), kThreads, 0, L->stream>>>(args); break;            \
    case 5: kern<5><<<(grid), kThreads, 0, L->stream>>>(args); break;            \
    default: kern<6><<<(grid), kThreads, 0, L->stream>>>(args); break;           \
  }

// the launches of one stage. step: a stage of SSP33!'s loop body with t and dt on the device
// (mode 2 / 1 of k_line_begin); otherwise a lone RHS at host time t with dt_set.
cudaError_t launch_stage(LineSolve* L, double t, int nstage, double dt_set, bool step) {
  const int flags = line_flags(L, nstage, step);
  LineArgs a = args_of(L, nstage, flags);
  const int grid = (L->K + kThreads - 1) / kThreads;
  const bool minent = (flags & LF_MINENT) && nstage == 1;
  if (step) {
    k_line_begin<<<1, 32, 0, L->stream>>>(a, nstage == 1 ? 2 : 1, 0.0, 0.0, minent ? 1 : 0);
  } else {
    // a lone RHS takes the dt it is given, except for the CFL's starting value
    const double dinit = host_jmin(L->prm.CFL * L->prm.dt0, L->prm.T - t);
    const double dkey = (flags & LF_CFL) ? dinit : dt_set;
    k_line_begin<<<1, 32, 0, L->stream>>>(a, 0, dkey, dt_set, (minent && t == L->prm.t0) ? 1 : 0);
  }
  L->launches += 1;
  if (line_layout(L) == P2DE_LAYOUT_TEAM) {
    switch (L->N1D) {
      case 2: k_line_face_team<2><<<L->K, kFaceTeamThreads, 0, L->stream>>>(a); break;
      case 3: k_line_face_team<3><<<L->K, kFaceTeamThreads, 0, L->stream>>>(a); break;
      case 4: k_line_face_team<4><<<L->K, kFaceTeamThreads, 0, L->stream>>>(a); break;
      case 5: k_line_face_team<5><<<L->K, kFaceTeamThreads, 0, L->stream>>>(a); break;
      default: k_line_face_team<6><<<L->K, kFaceTeamThreads, 0, L->stream>>>(a); break;
    }
  } else {
    LINE_LAUNCH(k_line_face, (2 * L->K + kThreads - 1) / kThreads, a);
  }
  L->launches += 1;
  if (flags & LF_LOW) {
    if (line_layout(L) == P2DE_LAYOUT_TEAM) {
      LINE_LAUNCH(k_line_low_team, (L->K + kTeamE - 1) / kTeamE, a);
    } else {
      LINE_LAUNCH(k_line_low, grid, a);
    }
    L->launches += 1;
  }
  if (minent) {  // gated on the device by the begin kernel's t == t0 test
    const long long nodes = (long long)L->K * L->N1D;
    k_line_phimin<<<(int)((nodes + 255) / 256), 256, 0, L->stream>>>(a);
    L->launches += 1;
  }
  if (flags & LF_HIGH) {
    const long long np = (long long)L->K * L->npair;
    k_line_pairs<<<(int)((np + kThreads - 1) / kThreads), kThreads, 0, L->stream>>>(a);
    if (line_layout(L) == P2DE_LAYOUT_TEAM) {
      LINE_LAUNCH(k_line_high_team, (L->K + kTeamE - 1) / kTeamE, a);
    } else {
      LINE_LAUNCH(k_line_high, grid, a);
    }
    L->launches += 2;
  }
  if (flags & (LF_SUBCELL | LF_UPDATE)) {
    if (line_layout(L) == P2DE_LAYOUT_TEAM) {
      LINE_LAUNCH(k_line_update_team, (L->K + kTeamE - 1) / kTeamE, a);
    } else {
      LINE_LAUNCH(k_line_update, grid, a);
    }
    L->launches += 1;
  }
  return cudaGetLastError();
}

// the launches of one SSP33! loop body on L->stream
cudaError_t enqueue_step(LineSolve* L) {
  cudaError_t e = cudaSuccess;
  for (int stage = 1; stage <= 3 && e == cudaSuccess; ++stage) e = launch_stage(L, 0.0, stage, 0.0, true);
  if (e != cudaSuccess) return e;
  k_line_end<<<1, 32, 0, L->stream>>>(args_of(L, 3, 0));
  L->launches += 1;
  return cudaGetLastError();
}

int check(LineSolve* L, std::string& err) {
  int st = 0;
  cudaError_t e = cudaMemcpyAsync(&st, L->status, sizeof(int), cudaMemcpyDeviceToHost, L->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(L->stream);
  if (e != cudaSuccess) {
    err = std::string("line solve: ") + cudaGetErrorString(e);
    return P2DE_ERR_CUDA;
  }
  if (st & (ST_NOT_POSITIVE | ST_NAN)) {
    err = "density or internal energy not positive (status " + std::to_string(st) + ")";
    return P2DE_ERR_NOT_POSITIVE;
  }
  if (st & ST_BAD_DT) {
    err = "time step not positive (status " + std::to_string(st) + ")";
    return P2DE_ERR_BAD_DT;
  }
  return P2DE_OK;
}

double read_dt(LineSolve* L, cudaError_t& e) {
  unsigned long long b = 0;
  e = cudaMemcpyAsync(&b, L->dtkey, sizeof b, cudaMemcpyDeviceToHost, L->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(L->stream);
  double d;
  std::memcpy(&d, &b, sizeof d);
  return d;
}

}  // namespace

int line_validate(const p2de_param* prm, const p2de_mesh* mesh, std::string& err) {
  if (prm->reference_semantics) {
    err = "CompressibleEulerIdealGas{Dim1}: the reference raises a MethodError in every RHS (Bx(::Dim1) "
          "calls reference_to_physical with dim last, rhs_utils.jl:18); use reference_semantics = 0";
    return P2DE_ERR_UNSUPPORTED;
  }
  if (prm->N < 1 || prm->N > 5 || prm->K < 1) {
    err = "N outside 1..5 or K < 1";
    return P2DE_ERR_INVALID_ARGUMENT;
  }
  if (prm->rhs_type < 0 || prm->rhs_type > 2 || prm->bound_type < 0 || prm->bound_type > 9 ||
      prm->shock_capture < 0 || prm->shock_capture > 1 || prm->rhs_limiter < 0 || prm->rhs_limiter > 1 ||
      prm->approximation_basis < 0 || prm->approximation_basis > 1 || prm->entropyproj_limiter < 0 ||
      prm->entropyproj_limiter > 1) {
    err = "rhs_type/bound_type/rhs_limiter/basis out of range";
    return P2DE_ERR_INVALID_ARGUMENT;
  }
  if ((prm->low_order_surface_flux != P2DE_FLUX_LAX_FRIEDRICHS_ON_NODAL_VAL &&
       prm->low_order_surface_flux != P2DE_FLUX_LAX_FRIEDRICHS_ON_PROJECTED_VAL) ||
      prm->high_order_surface_flux != P2DE_FLUX_LAX_FRIEDRICHS_ON_PROJECTED_VAL) {
    err = "surface fluxes: LaxFriedrichsOnNodalVal or LaxFriedrichsOnProjectedVal";
    return P2DE_ERR_UNSUPPORTED;
  }
  if (prm->precision != P2DE_PRECISION_FP64 || mesh->nW || mesh->nS) {
    err = "CompressibleEulerIdealGas{Dim1}: FP64, periodic, inflow and outflow faces";
    return P2DE_ERR_UNSUPPORTED;
  }
  const int b = prm->bound_type;
  if (prm->approximation_basis == P2DE_BASIS_GAUSS && prm->rhs_limiter == P2DE_LIMITER_SUBCELL &&
      prm->rhs_type == P2DE_RHS_ES_LIMITED_LOW_ORDER_POS &&
      is_one_of(b, {P2DE_BOUND_POSITIVITY_AND_CELL_ENTROPY, P2DE_BOUND_TVD_AND_CELL_ENTROPY,
                    P2DE_BOUND_POSITIVITY_AND_RELAXED_CELL_ENTROPY, P2DE_BOUND_TVD_AND_RELAXED_CELL_ENTROPY})) {
    err = "CompressibleEulerIdealGas{Dim1}: no cell-entropy bounds on Gauss nodes (enforce_ES_subcell_interface! "
          "has no Dim1 method for GaussCollocation, subcell.jl:755-759)";
    return P2DE_ERR_UNSUPPORTED;
  }
  const int64_t nfk = 2 * (int64_t)prm->K;
  if (!mesh->geom || !mesh->mapP) {
    err = "geom and mapP are required";
    return P2DE_ERR_INVALID_ARGUMENT;
  }
  for (int64_t i = 0; i < nfk; ++i)
    if (mesh->mapP[i] < 1 || mesh->mapP[i] > nfk) {
      err = "mapP[" + std::to_string(i) + "] out of 1.." + std::to_string(nfk);
      return P2DE_ERR_INVALID_ARGUMENT;
    }
  auto list_ok = [&](const int64_t* m, int64_t cnt) {
    if (cnt < 0 || (cnt > 0 && !m)) return false;
    for (int64_t i = 0; i < cnt; ++i)
      if (m[i] < 1 || m[i] > nfk) return false;
    return true;
  };
  if (!list_ok(mesh->mapI, mesh->nI) || !list_ok(mesh->mapO, mesh->nO) || (mesh->nI > 0 && !mesh->Ival)) {
    err = "mapI/mapO/Ival: bad list";
    return P2DE_ERR_INVALID_ARGUMENT;
  }
  for (int k = 0; k < prm->K; ++k)
    if (!(mesh->geom[5 * (size_t)k] > 0.0)) {
      err = "J[" + std::to_string(k) + "] is not positive";
      return P2DE_ERR_INVALID_ARGUMENT;
    }
  return P2DE_OK;
}

int line_create(const p2de_param* prm, const p2de_mesh* mesh, cudaStream_t st, LineSolve** out, std::string& err) {
  *out = nullptr;
  const int rc = line_validate(prm, mesh, err);
  if (rc != P2DE_OK) return rc;
  const int K = prm->K, n = prm->N + 1;
  const int64_t nfk = 2 * (int64_t)K;
  LineOps ops;
  if (build_line_ops(prm->N, prm->ZEROTOL, &ops, prm->approximation_basis) != 0) {
    err = "Line operators: degree out of range";
    return P2DE_ERR_INVALID_ARGUMENT;
  }
  auto* L = new LineSolve();
  L->prm = *prm;
  L->N1D = n;
  L->K = K;
  L->npair = ops.npair;
  L->stream = st;
  std::vector<int32_t> nbr(nfk), bcidx(nfk, 0);
  std::vector<int8_t> bc(nfk, BC_INTERIOR);
  for (int64_t i = 0; i < nfk; ++i) nbr[i] = (int32_t)(mesh->mapP[i] - 1);
  for (int64_t i = 0; i < mesh->nI; ++i) {
    bc[mesh->mapI[i] - 1] = BC_INFLOW;
    bcidx[mesh->mapI[i] - 1] = (int32_t)i;
  }
  for (int64_t i = 0; i < mesh->nO; ++i) bc[mesh->mapO[i] - 1] = BC_OUTFLOW;
  const size_t nq = (size_t)4 * n * K;
  cudaError_t e = cudaSuccess;
  auto A = [&](auto** p, size_t cnt) {
    if (e == cudaSuccess) e = dalloc(L, p, cnt);
  };
  A(&L->Uq, nq);
  A(&L->resW, nq);
  A(&L->rhsL, nq);
  A(&L->rhsH, nq);
  A(&L->rhsU, nq);
  A(&L->BFL, (size_t)8 * K);
  A(&L->BFH, (size_t)8 * K);
  A(&L->uf, (size_t)8 * K);
  A(&L->theta, (size_t)3 * 2 * K);
  A(&L->Lloc, (size_t)3 * 2 * n * K);
  A(&L->Lraw, (size_t)2 * n * K);
  A(&L->fbar, (size_t)8 * (n + 1) * K);
  A(&L->Lelem, (size_t)3 * K);
  A(&L->sf, (size_t)4 * kLineMaxPairs * K);
  A(&L->geom, (size_t)5 * K);
  A(&L->Ival, (size_t)3 * (mesh->nI > 0 ? mesh->nI : 1));
  A(&L->phimin, 1);
  A(&L->nbr, (size_t)nfk);
  A(&L->bcidx, (size_t)nfk);
  A(&L->bc, (size_t)nfk);
  A(&L->dtkey, 2);
  A(&L->minrec, 6);
  A(&L->ts, TS_N);
  A(&L->status, 1);
  A(&L->ops, 1);
  auto up = [&](void* dst, const void* src, size_t bytes) {
    if (e == cudaSuccess) e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st);
  };
  up(L->geom, mesh->geom, sizeof(double) * 5 * K);
  if (mesh->nI > 0) up(L->Ival, mesh->Ival, sizeof(double) * 3 * mesh->nI);
  up(L->nbr, nbr.data(), sizeof(int32_t) * nfk);
  up(L->bcidx, bcidx.data(), sizeof(int32_t) * nfk);
  up(L->bc, bc.data(), (size_t)nfk);
  up(L->ops, &ops, sizeof ops);
  // zeros(Float64, 1) of s_modified_min until t == t0 at stage 1
  long long k0 = 0;  // the ordered key of +0.0
  up(L->phimin, &k0, sizeof k0);
  std::vector<double> ones((size_t)3 * 2 * K, 1.0);
  up(L->theta, ones.data(), sizeof(double) * ones.size());
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    err = std::string("Line setup: ") + cudaGetErrorString(e);
    line_destroy(L);
    return P2DE_ERR_CUDA;
  }
  *out = L;
  return P2DE_OK;
}

void line_destroy(LineSolve* L) {
  if (!L) return;
  if (L->stream) cudaStreamSynchronize(L->stream);
  if (L->graph) cudaGraphExecDestroy(L->graph);
  for (void* p : L->allocs) cudaFree(p);
  delete L;
}

int64_t line_field_count(const LineSolve* L, int field) {
  const int64_t n = L->N1D, K = L->K;
  switch (field) {
    case P2DE_FIELD_UQ:
    case P2DE_FIELD_RHSU:
    case P2DE_FIELD_RHSL:
    case P2DE_FIELD_RHSH:
    case P2DE_FIELD_RESW:
    case P2DE_FIELD_RHSXYL:
    case P2DE_FIELD_RHSXYH: return 3 * n * K;
    case P2DE_FIELD_BF_L:
    case P2DE_FIELD_BF_H: return 3 * 2 * K;
    case P2DE_FIELD_L_LOCAL: return 2 * n * K;
    case P2DE_FIELD_L: return K;
    case P2DE_FIELD_THETA_LOCAL: return 2 * K;
    default: return -1;
  }
}

int line_set_Uq(LineSolve* L, const double* Uq, std::string& err) {
  const size_t nodes = (size_t)L->N1D * L->K;
  std::vector<double> full(4 * nodes);
  for (size_t i = 0; i < nodes; ++i) {
    full[4 * i] = Uq[3 * i];
    full[4 * i + 1] = Uq[3 * i + 1];
    full[4 * i + 2] = 0.0;
    full[4 * i + 3] = Uq[3 * i + 2];
  }
  cudaError_t e = cudaMemcpyAsync(L->Uq, full.data(), sizeof(double) * full.size(), cudaMemcpyHostToDevice, L->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(L->status, 0, sizeof(int), L->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(L->stream);
  if (e != cudaSuccess) {
    err = std::string("set_Uq: ") + cudaGetErrorString(e);
    return P2DE_ERR_CUDA;
  }
  return P2DE_OK;
}

int line_get_field(LineSolve* L, int field, int nstage, double* out, std::string& err) {
  const int64_t cnt = line_field_count(L, field);
  if (cnt < 0) return P2DE_ERR_INVALID_ARGUMENT;
  const bool staged = field == P2DE_FIELD_L_LOCAL || field == P2DE_FIELD_L || field == P2DE_FIELD_THETA_LOCAL;
  if (staged && (nstage < 1 || nstage > 3)) return P2DE_ERR_INVALID_ARGUMENT;
  const double* src = nullptr;
  bool states = true;
  switch (field) {
    case P2DE_FIELD_UQ: src = L->Uq; break;
    case P2DE_FIELD_RHSU: src = L->rhsU; break;
    case P2DE_FIELD_RHSL:
    case P2DE_FIELD_RHSXYL: src = L->rhsL; break;
    case P2DE_FIELD_RHSH:
    case P2DE_FIELD_RHSXYH: src = L->rhsH; break;
    case P2DE_FIELD_RESW: src = L->resW; break;
    case P2DE_FIELD_BF_L: src = L->BFL; break;
    case P2DE_FIELD_BF_H: src = L->BFH; break;
    case P2DE_FIELD_L_LOCAL: src = L->Lloc + cnt * (nstage - 1), states = false; break;
    case P2DE_FIELD_L: src = L->Lelem + cnt * (nstage - 1), states = false; break;
    case P2DE_FIELD_THETA_LOCAL: src = L->theta + cnt * (nstage - 1), states = false; break;
  }
  cudaError_t e;
  if (states) {  // four slots per state -> (rho, rhou, E)
    std::vector<double> full((size_t)cnt / 3 * 4);
    e = cudaMemcpyAsync(full.data(), src, sizeof(double) * full.size(), cudaMemcpyDeviceToHost, L->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(L->stream);
    for (int64_t i = 0; i < cnt / 3; ++i) {
      out[3 * i] = full[4 * i];
      out[3 * i + 1] = full[4 * i + 1];
      out[3 * i + 2] = full[4 * i + 3];
    }
  } else {
    e = cudaMemcpyAsync(out, src, sizeof(double) * cnt, cudaMemcpyDeviceToHost, L->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(L->stream);
  }
  if (e != cudaSuccess) {
    err = std::string("get_field: ") + cudaGetErrorString(e);
    return P2DE_ERR_CUDA;
  }
  return P2DE_OK;
}

int line_rhs(LineSolve* L, double t, double dt, int nstage, double* dt_out, std::string& err) {
  if (nstage < 1 || nstage > 3) return P2DE_ERR_INVALID_ARGUMENT;
  cudaError_t e = launch_stage(L, t, nstage, dt, false);
  if (e != cudaSuccess) {
    err = std::string("line rhs: ") + cudaGetErrorString(e);
    return P2DE_ERR_CUDA;
  }
  const double d = read_dt(L, e);
  if (e != cudaSuccess) {
    err = std::string("line rhs: ") + cudaGetErrorString(e);
    return P2DE_ERR_CUDA;
  }
  if (dt_out) *dt_out = d;
  return check(L, err);
}

namespace {

// sets the device time, runs `nsteps` loop bodies (one CUDA graph replayed), reads back the
// time state and the status word once
int run_steps(LineSolve* L, double* t, int64_t nsteps, double ts_out[TS_N], std::string& err) {
  cudaError_t e = cudaMemcpyAsync(L->ts + TS_T, t, sizeof(double), cudaMemcpyHostToDevice, L->stream);
  if (e == cudaSuccess && nsteps > 1 && !L->graph) {  // capture one body on a private stream
    cudaStream_t cap, user = L->stream;
    e = cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking);
    if (e == cudaSuccess) {
      cudaGraph_t g = nullptr;
      const int64_t before = L->launches;
      L->stream = cap;
      e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
      const cudaError_t e1 = e == cudaSuccess ? enqueue_step(L) : e;
      const cudaError_t e2 = e == cudaSuccess ? cudaStreamEndCapture(cap, &g) : e;
      L->stream = user;
      L->launches = before;
      cudaStreamDestroy(cap);
      e = e1 != cudaSuccess ? e1 : e2;
      if (e == cudaSuccess) e = cudaGraphInstantiate(&L->graph, g, 0);
      if (g) cudaGraphDestroy(g);
    }
  }
  for (int64_t i = 0; i < nsteps && e == cudaSuccess; ++i) {
    if (L->graph) {
      e = cudaGraphLaunch(L->graph, L->stream);
      L->launches += line_step_launches(L);
    } else {
      e = enqueue_step(L);
    }
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(ts_out, L->ts, sizeof(double) * TS_N, cudaMemcpyDeviceToHost, L->stream);
  if (e != cudaSuccess) {
    err = std::string("line steps: ") + cudaGetErrorString(e);
    return P2DE_ERR_CUDA;
  }
  const int rc = check(L, err);  // synchronizes
  *t = ts_out[TS_T];
  return rc;
}

}  // namespace

int line_step(LineSolve* L, double* t, double* dt_out, std::string& err) {
  double ts[TS_N];
  double tt = *t;
  const int rc = run_steps(L, &tt, 1, ts, err);
  if (rc != P2DE_OK) return rc;
  const bool stepped = ts[TS_DONE] == 0.0;
  if (dt_out) *dt_out = stepped ? ts[TS_DT] : 0.0;
  if (stepped) *t = tt;
  return P2DE_OK;
}

int line_advance(LineSolve* L, int64_t nsteps, double* t, int64_t* steps_done, double* dt_last, std::string& err) {
  double ts[TS_N];
  cudaError_t e = cudaMemcpyAsync(ts, L->ts, sizeof ts, cudaMemcpyDeviceToHost, L->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(L->stream);
  if (e != cudaSuccess) {
    err = std::string("line advance: ") + cudaGetErrorString(e);
    return P2DE_ERR_CUDA;
  }
  const double steps0 = ts[TS_STEPS];
  const int rc = run_steps(L, t, nsteps, ts, err);
  if (steps_done) *steps_done = (int64_t)(ts[TS_STEPS] - steps0);
  if (dt_last) *dt_last = ts[TS_DT];
  return rc;
}

int line_layout(const LineSolve* L) {
  if (L->layout >= 0) return L->layout;
  return L->K < kTeamMaxK ? P2DE_LAYOUT_TEAM : P2DE_LAYOUT_FLAT;
}

int line_set_layout(LineSolve* L, int layout, std::string& err) {
  if (layout != P2DE_LAYOUT_FLAT && layout != P2DE_LAYOUT_TEAM) {
    err = "a Line solve takes P2DE_LAYOUT_FLAT or P2DE_LAYOUT_TEAM, not " + std::to_string(layout);
    return P2DE_ERR_INVALID_ARGUMENT;
  }
  cudaError_t e = cudaStreamSynchronize(L->stream);
  if (e != cudaSuccess) {
    err = cudaGetErrorString(e);
    return P2DE_ERR_CUDA;
  }
  L->layout = layout;
  if (L->graph) {  // the captured step holds the old kernel
    cudaGraphExecDestroy(L->graph);
    L->graph = nullptr;
  }
  return P2DE_OK;
}

int line_step_launches(const LineSolve* L) {
  int c = 1;  // k_line_end
  for (int stage = 1; stage <= 3; ++stage) {
    const int f = line_flags(L, stage, true);
    c += 1 + 1 + ((f & LF_LOW) ? 1 : 0) + ((f & LF_MINENT) && stage == 1 ? 1 : 0) + ((f & LF_HIGH) ? 2 : 0) + 1;
  }
  return c;
}

}  // namespace p2de
