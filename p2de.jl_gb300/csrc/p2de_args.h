// Launch arguments shared by the host code and the stage kernels.
#pragma once

#include <cmath>

#include <stdint.h>

#include "p2de_tables.h"

namespace p2de {

// flag bits of StageArgs::flags
enum : int {
  F_DO_LOW = 1 << 0,        // low-order graph-viscosity RHS
  F_DO_HIGH = 1 << 1,       // high-order ES flux differencing RHS
  F_DO_LIMIT = 1 << 2,      // subcell limiter
  F_WRITE_DEBUG = 1 << 3,   // write rhsxyL/H, BF_L/H, rhsL, rhsH to global
  F_AXIS_ALIGNED = 1 << 4,  // all elements have sxJ = ryJ = 0
  F_REF_SEM = 1 << 5,       // reference 4-name destructuring of the 5-tuple bound
  F_CELL_ENTROPY = 1 << 6,  // PositivityAndCellEntropyBound
  F_UPDATE = 1 << 7,        // stage kernel B applies the SSP-RK3 stage update
  F_RHSU_FROM_L = 1 << 8,   // rhsU = rhsL (LowOrderPositivity)
  F_RHSU_FROM_H = 1 << 9,   // rhsU = rhsH (FluxDiffRHS)
  F_CFL = 1 << 10,          // stage 1: low-order positivity CFL reduction
  F_ACC64 = 1 << 11,        // FP32 kernel: pair fluxes gathered and lifted in FP64
  F_TVD = 1 << 12,          // TVD density bounds from the low-order densities in rhoL
  F_LOW_ONLY = 1 << 13,     // kernel A stops after the low-order RHS and stores rhoL
  F_SHOCK = 1 << 14,        // HennemannShockCapture blending factor caps the subcell factors
  F_ZHANG_SHU = 1 << 15,    // ZhangShuLimiter: one factor per element, rhsU written by kernel A
  F_MIN_ENTROPY = 1 << 16,  // min-entropy bounds: bisection for phi >= Lphi - POSTOL
  F_RELAXED = 1 << 17,      // relaxed bounds: smoothness factor from the modal energies
  F_GAUSS = 1 << 18,        // GaussCollocation: projected face states, face pairs, Vf lift
  F_EPROJ = 1 << 19,        // NodewiseScaledExtrapolation: theta per face node
  F_KPP = 1 << 20,          // KPP{Dim2}: the scalar in component 0, the others 0
  F_LFPROJ = 1 << 21        // LaxFriedrichsOnProjectedVal low-order flux: its CFL term
};
// the modes whose branches only the EXT instantiation of stage kernel A compiles
constexpr int kExtFlags = F_ZHANG_SHU | F_MIN_ENTROPY | F_RELAXED | F_GAUSS | F_EPROJ | F_KPP | F_LFPROJ;

// boundary codes per face node
enum : int8_t { BC_INTERIOR = 0, BC_INFLOW = 1, BC_OUTFLOW = 2, BC_WALL = 3, BC_SHOCK = 4 };

// device scalar slots
enum : int { S_T = 0, S_DT_LIM = 1, S_DT = 2, S_DONE = 3, S_STEPS = 4, S_NSCAL = 8 };

// status bits
enum : int { ST_NOT_POSITIVE = 1, ST_BAD_DT = 2, ST_NAN = 4 };

struct StageArgs {
  int K;
  int nstage;  // 1..3
  int flags;
  int epb;  // elements per block (<= the degree's maximum, Cfg::E_MAX)
  // thread layout of the high-order pair and gather phases (p2de_layout): 0 flat (element,
  // pair) and (element, node) loops; 1 whole lines per warp on axis-aligned LGL elements
  int layout;
  // threads per block of stage kernel A (a multiple of 32 up to Cfg::THREADS; 0: Cfg::THREADS)
  int threads;
  const OpTable* ops;
  double* Uq;
  double* resW;
  const double* geom;     // K x 5: J, rxJ, sxJ, ryJ, syJ
  const int32_t* nbr;     // Nfp x K: 0-based exterior face-node linear index (mapP - 1)
  const int8_t* bc;       // Nfp x K boundary code
  const int32_t* bcidx;   // Nfp x K index into Ival / xyS
  const double* Ival;     // nI x 4
  const double* xyS;      // nS x 2
  double shock_x0, shock_inv_slope, shock_speed;
  double shock_post[4], shock_pre[4];
  double gamma, gm1, CFL, dt0, T, zeta, ZEROTOL;
  double* rhsL;
  double* rhsH;
  double* rhsU;
  double* rhsxyL;
  double* rhsxyH;
  double* BFL;
  double* BFH;
  double* fbar;  // K x (2 dirs x 2 (H, L) x NSF x 4)
  double* Lpre;  // K x 2 x (Nq+N1D), before symmetrization
  double* Lfin;  // 3 stages x K x 2 x (Nq+N1D)
  double* scal;  // S_* slots
  unsigned long long* dtmin_bits;
  long long* minrec;  // 3 stages x {min rho, min rhoe} as ordered keys
  int* status;
  unsigned long long* counters;  // [0] quadratic rhoe solves evaluated by the bound phase
  double* rhoL;  // K x Nq low-order densities U + dt rhsL (TVD bounds only)
  const double* geomx;  // K x 16 geometry factors (geom_factor), or null: computed per launch
  double sc_TN, sc_q;   // HennemannShockCapture: TN and -log((1-1e-4)/1e-4) / TN
  double* Lelem;        // 3 stages x K: ZhangShuLimiter factors (F_ZHANG_SHU)
  double* phimin;       // [0]: min of phi = rhoe rho^-gamma over the state at t0, stage 1
  double t0, POSTOL;
  double s0;            // log10(N^-4), the centre of the smoothness ramp (subcell.jl:944)
  double beta;          // relaxed cell-entropy bounds: target scale 1 - beta eps_k
  double* ufproj;       // K x Nfp x 4: entropy-projected face states (GaussCollocation)
  double* theta;        // 3 stages x K x Nfp: entropy-projection limiting factors
  double eta;           // LimitingParameter eta (bounds of the projected face states)
};

// StageArgs shock-capture constants of update_blending_factor! (shock_capture.jl:123-126)
inline void set_shock_capture(StageArgs& a, int N, double sc_a, double sc_c) {
  const double TN = sc_a * std::pow(10.0, -sc_c * std::pow((double)(N + 1), 0.25));
  const double alphaE0 = 0.0001;
  const double s_factor = std::log((1 - alphaE0) / alphaE0);
  a.sc_TN = TN;
  a.sc_q = -s_factor / TN;
}

// flag bits of a SubcellLimiter bound type (p2de_bound_type, Solver.jl:47-62)
inline int bound_flags(int bound_type) {
  switch (bound_type) {
    case 1: return F_CELL_ENTROPY;                            // PositivityAndCellEntropyBound
    case 2: return F_TVD;                                     // TVDBound
    case 3: return F_TVD | F_CELL_ENTROPY;                    // TVDAndCellEntropyBound
    case 4: return F_MIN_ENTROPY;                             // PositivityAndMinEntropyBound
    case 5: return F_MIN_ENTROPY | F_RELAXED;                 // PositivityAndRelaxedMinEntropyBound
    case 6: return F_CELL_ENTROPY | F_RELAXED;                // PositivityAndRelaxedCellEntropyBound
    case 7: return F_TVD | F_MIN_ENTROPY;                     // TVDAndMinEntropyBound
    case 8: return F_TVD | F_MIN_ENTROPY | F_RELAXED;         // TVDAndRelaxedMinEntropyBound
    case 9: return F_TVD | F_CELL_ENTROPY | F_RELAXED;        // TVDAndRelaxedCellEntropyBound
    default: return 0;                                        // PositivityBound
  }
}

// StageArgs constants of the min-entropy and relaxed bounds: t0 (the stage at which the
// initial minimum of phi is taken), POSTOL, s0 = log10(N^-4) (subcell.jl:944, with N^-4
// as Float64(N)^-4) and the relaxed cell-entropy beta
inline void set_bound_constants(StageArgs& a, int N, double t0, double POSTOL, double beta) {
  a.t0 = t0;
  a.POSTOL = POSTOL;
  a.s0 = std::log(1.0 / ((double)N * N * N * N)) / std::log(10.0);
  a.beta = beta;
}

}  // namespace p2de
