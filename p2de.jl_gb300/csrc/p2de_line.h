// CompressibleEulerIdealGas{Dim1} on a Line mesh: device state and host driver of the
// RHS and SSP-RK3 stage (p2de_line.cu). Reached through the p2de_* entry points when
// param.equation is P2DE_EQUATION_COMPRESSIBLE_EULER_1D.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/p2de.h"
#include "p2de_tables.h"

namespace p2de {

struct LineSolve {
  p2de_param prm{};
  int N1D = 0, K = 0;
  cudaStream_t stream = nullptr;
  // states hold four slots per node, (rho, rhou, 0, E), like the Dim2 layout
  double *Uq = nullptr, *resW = nullptr, *rhsL = nullptr, *rhsH = nullptr, *rhsU = nullptr;
  double *BFL = nullptr, *BFH = nullptr;  // 2 x 4 per element (the x part)
  double *uf = nullptr;                   // projected face states u_tilde, 2 x 4 per element
  double *theta = nullptr;                // theta_local, 3 stages x K x 2
  double *Lloc = nullptr;                 // L_local, 3 stages x K x 2 N1D
  double *Lraw = nullptr;                 // L_local before symmetrization, K x 2 N1D
  double *fbar = nullptr;                 // f_bar_H, f_bar_L: K x 2 x (N1D+1) x 4
  double *Lelem = nullptr;                // ZhangShuLimiter L, 3 stages x K
  double *sf = nullptr;                   // volume two-point terms S fS, K x kLineMaxPairs x 4
  int npair = 0;                          // nonzero pairs of Srh_db per element
  int layout = -1;                        // P2DE_LAYOUT_FLAT or _TEAM; -1: by the element count
  double *geom = nullptr, *Ival = nullptr, *phimin = nullptr;
  int32_t *nbr = nullptr, *bcidx = nullptr;
  int8_t* bc = nullptr;
  unsigned long long* dtkey = nullptr;  // bits of the step's dt (positive: ordered) and of the limiter's dt
  long long* minrec = nullptr;          // min rho, min rhoe per stage (ordered keys)
  double* ts = nullptr;                 // device time state: t, dt, done, steps, phi flag
  cudaGraphExec_t graph = nullptr;      // one SSP-RK3 step, replayed by line_advance
  int* status = nullptr;
  LineOps* ops = nullptr;
  int64_t launches = 0;
  std::vector<void*> allocs;
};

// host-side checks of a Dim1 descriptor (no device needed)
int line_validate(const p2de_param* prm, const p2de_mesh* mesh, std::string& err);
int line_create(const p2de_param* prm, const p2de_mesh* mesh, cudaStream_t st, LineSolve** out, std::string& err);
void line_destroy(LineSolve* L);
int64_t line_field_count(const LineSolve* L, int field);
int line_set_Uq(LineSolve* L, const double* Uq, std::string& err);
int line_get_field(LineSolve* L, int field, int nstage, double* out, std::string& err);
// rhs!(state, solver, state_param, TimeParam(t, dt, nstage)) without the stage update
int line_rhs(LineSolve* L, double t, double dt, int nstage, double* dt_out, std::string& err);
// one SSP33! loop body from *t
int line_step(LineSolve* L, double* t, double* dt_out, std::string& err);
// nsteps loop bodies from *t with t and dt on the device (a captured step replayed); steps
// after the final time are no-ops
int line_advance(LineSolve* L, int64_t nsteps, double* t, int64_t* steps_done, double* dt_last, std::string& err);
// kernel launches of one step
int line_step_launches(const LineSolve* L);
// the layout of the high-order and limiter kernel: P2DE_LAYOUT_FLAT (one thread per element)
// or P2DE_LAYOUT_TEAM (a team of lanes per element); the default follows the element count
int line_set_layout(LineSolve* L, int layout, std::string& err);
int line_layout(const LineSolve* L);

}  // namespace p2de
