/*
 * p2de.h — C ABI of the GB300 implementation of P2DE.jl's 2D compressible-Euler
 * DG right-hand side and SSP-RK3 time step (libp2de_gpu.so).
 *
 * Every entry point returns an int status (p2de_status); no exception crosses the
 * ABI. Host buffers are caller-owned and copied; device memory is owned by the
 * solver handle. One handle is used from one host thread at a time.
 *
 * Array layouts are those of P2DE.jl (column-major Julia arrays):
 *   SVector{4} array A[i,k]            -> A[c + 4*(i + n*k)]          (c = component)
 *   SVector{2,SVector{4}} array B[i,k] -> B[c + 4*(d + 2*(i + n*k))]  (d = x,y)
 *   L_local[i,d,k] (one stage)         -> L[i + (Nq+N1D)*(d + 2*k)]
 * Node order inside an element is tensor-product GLL with r fastest,
 * i = ir + (N+1)*is; face nodes are ordered by faces r=-1, r=+1, s=-1, s=+1,
 * each along the face's tangential coordinate (StartUpDG's Quad convention).
 * Julia passes reinterpret(Float64, Uq), which is bitwise this layout.
 */
#ifndef P2DE_H
#define P2DE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define P2DE_ABI_VERSION 5

typedef enum p2de_status {
  P2DE_OK = 0,
  P2DE_ERR_INVALID_ARGUMENT = 1, /* bad sizes, null pointers, unsupported N */
  P2DE_ERR_UNSUPPORTED = 2,      /* method combination not built */
  P2DE_ERR_CUDA = 3,             /* CUDA runtime error; see p2de_last_error */
  P2DE_ERR_OUT_OF_MEMORY = 4,
  P2DE_ERR_NOT_POSITIVE = 5,     /* density or internal energy <= 0 or NaN in the state */
  P2DE_ERR_BAD_DT = 6,           /* time step <= 0 or NaN */
  P2DE_ERR_NO_DEVICE = 7,        /* no CUDA device visible */
  P2DE_ERR_BUDGET = 8,           /* serving: request larger than the HBM budget */
  P2DE_ERR_NOT_FOUND = 9         /* serving: unknown request id */
} p2de_status;

/* RHS dispatch types (src/common/types/Solver.jl:1-36). */
typedef enum p2de_rhs_type {
  P2DE_RHS_ES_LIMITED_LOW_ORDER_POS = 0, /* LimitedDG with ChandrashekarFlux volume flux */
  P2DE_RHS_LOW_ORDER_POSITIVITY = 1,     /* LowOrderPositivity */
  P2DE_RHS_ENTROPY_STABLE = 2            /* FluxDiffRHS{ChandrashekarFlux} */
} p2de_rhs_type;

/* Subcell limiter bounds (Solver.jl:47-54). */
typedef enum p2de_bound_type {
  P2DE_BOUND_POSITIVITY = 0,                  /* PositivityBound */
  P2DE_BOUND_POSITIVITY_AND_CELL_ENTROPY = 1, /* PositivityAndCellEntropyBound */
  P2DE_BOUND_TVD = 2,                         /* TVDBound (subcell.jl:112-141): density in the
                                                 min/max of the low-order density over the
                                                 node and its low_order_stencil */
  P2DE_BOUND_TVD_AND_CELL_ENTROPY = 3,        /* TVDAndCellEntropyBound */
  /* modified specific entropy phi = rhoe rho^(-gamma) >= Lphi - POSTOL by bisection
     (limiter_utils.jl:19-24,43-50), Lphi the min of phi over the node and its
     low_order_stencil (subcell.jl:53-72) */
  P2DE_BOUND_POSITIVITY_AND_MIN_ENTROPY = 4,          /* PositivityAndMinEntropyBound */
  P2DE_BOUND_POSITIVITY_AND_RELAXED_MIN_ENTROPY = 5,  /* ...RelaxedMinEntropyBound: Lphi blended
                                                         with the global initial min of phi by
                                                         the smoothness factor (subcell.jl:937-956) */
  P2DE_BOUND_POSITIVITY_AND_RELAXED_CELL_ENTROPY = 6, /* ...RelaxedCellEntropyBound(beta): entropy
                                                         target scaled by 1 - beta eps_k (:750-753) */
  P2DE_BOUND_TVD_AND_MIN_ENTROPY = 7,                 /* TVDAndMinEntropyBound */
  P2DE_BOUND_TVD_AND_RELAXED_MIN_ENTROPY = 8,         /* TVDAndRelaxedMinEntropyBound */
  P2DE_BOUND_TVD_AND_RELAXED_CELL_ENTROPY = 9         /* TVDAndRelaxedCellEntropyBound(beta) */
} p2de_bound_type;

/* Equations (Solver.jl:97-121). KPP{Dim2} (src/math/KPP.jl) is the scalar rotating-wave
 * law u_t + (sin u)_x + (cos u)_y = 0 with wavespeed 1; its state arrays have one
 * component per node (Nc = 1, p2de_solver_field_count), on LGL nodes, with the subcell
 * limiter's factor equal to the shock-capture blending factor (subcell.jl:389-402). */
/* CompressibleEulerIdealGas{Dim1}(gamma) (Solver.jl:97-121, compressible_Navier_Stokes.jl
 * Dim1 methods) on a line of K elements: Nq = N+1 nodes and Nfp = 2 face nodes (r = -1, +1)
 * per element, states (rho, rhou, E) (Nc = 3), mesh geom rows (J, rxJ, 0, 0, 0), Ival nI x 3.
 * The reference's own Dim1 path does not run: Bx(::Dim1) passes its arguments to
 * reference_to_physical in the wrong order (rhs_utils.jl:18), a MethodError in every RHS.
 * With reference_semantics = 1 the solver is therefore refused (P2DE_ERR_UNSUPPORTED); with 0
 * it runs the Dim1 methods with their evident meaning: Bx = Br rxJ; the subcell bound from
 * rho_bound(dim, ...) (subcell.jl:225-237); N entries of dvdf per element (State.jl:184 sizes
 * them Nq - N1D = 0); and the element-boundary factors symmetrized across mapP with the last
 * used subcell face Nq+1 (subcell.jl:405-415 pairs index `end` = 2 N1D of element k-1 mod K). */
typedef enum p2de_equation {
  P2DE_EQUATION_COMPRESSIBLE_EULER = 0,   /* CompressibleEulerIdealGas{Dim2}(gamma) */
  P2DE_EQUATION_KPP = 1,                  /* KPP{Dim2}() */
  P2DE_EQUATION_COMPRESSIBLE_EULER_1D = 2 /* CompressibleEulerIdealGas{Dim1}(gamma) */
} p2de_equation;

/* Approximation bases (Solver.jl:38-40): collocation on the tensor-product LGL nodes, or
 * on the Gauss nodes with extrapolation to the face Gauss points (init.jl:83-131). */
typedef enum p2de_basis {
  P2DE_BASIS_LOBATTO = 0,  /* LobattoCollocation */
  P2DE_BASIS_GAUSS = 1     /* GaussCollocation */
} p2de_basis;

/* Entropy-projection limiters (Solver.jl:41-43): Gauss faces take the entropy variables
 * extrapolated by theta Vf + (1 - theta) Vf_low, theta per face node from the bounds of
 * filter.jl:91-130 by bisection. */
typedef enum p2de_entropyproj_limiter {
  P2DE_ENTROPYPROJ_NONE = 0,                       /* NoEntropyProjectionLimiter */
  P2DE_ENTROPYPROJ_NODEWISE_SCALED_EXTRAPOLATION = 1 /* NodewiseScaledExtrapolation */
} p2de_entropyproj_limiter;

/* RHS limiters (Solver.jl:72-91). */
typedef enum p2de_rhs_limiter {
  P2DE_LIMITER_SUBCELL = 0,   /* SubcellLimiter(bound, shockcapture) */
  P2DE_LIMITER_ZHANG_SHU = 1  /* ZhangShuLimiter(shockcapture): one factor per element from
                                 the positivity bounds at its nodes (zhangshu.jl:4-45);
                                 bound_type is not read */
} p2de_rhs_limiter;

/* Surface flux types (Solver.jl:19-22). Low order: LaxFriedrichsOnNodalVal or
 * LaxFriedrichsOnProjectedVal (the entropy-projected face states; its CFL adds
 * alpha lambdaB + |B| ws / 2 per face, low_order_graph_viscosity.jl:245-318); high order:
 * LaxFriedrichsOnProjectedVal. */
typedef enum p2de_surface_flux {
  P2DE_FLUX_LAX_FRIEDRICHS_ON_NODAL_VAL = 0,
  P2DE_FLUX_LAX_FRIEDRICHS_ON_PROJECTED_VAL = 1
} p2de_surface_flux;

typedef enum p2de_precision {
  P2DE_PRECISION_FP64 = 0, /* everything in FP64 */
  P2DE_PRECISION_MIXED = 1, /* volume flux differencing in FP32 with FP32
                               accumulation; low order, limiter, RK in FP64 */
  P2DE_PRECISION_MIXED_ACC64 = 2 /* volume two-point fluxes in FP32, their gather and
                                    lift accumulated in FP64 (a pair's term then cancels
                                    exactly between its two nodes); the rest as MIXED */
} p2de_precision;

/* Param (Solver.jl:151-170) flattened; method choices as enums. */
typedef struct p2de_param {
  int32_t N;       /* polynomial degree, 1..5 */
  int32_t K;       /* number of elements */
  double gamma;    /* CompressibleEulerIdealGas{Dim2}(gamma) */
  double POSTOL;   /* GlobalConstant */
  double ZEROTOL;
  double zeta;     /* LimitingParameter */
  double eta;
  double CFL;      /* TimesteppingParameter */
  double dt0;
  double t0;
  double T;
  int32_t rhs_type;                /* p2de_rhs_type */
  int32_t bound_type;              /* p2de_bound_type */
  int32_t low_order_surface_flux;  /* p2de_surface_flux */
  int32_t high_order_surface_flux; /* p2de_surface_flux */
  /* 1: reproduce limiter_utils.jl:66-70 exactly, where the 5-tuple bound
   * (Lrho, Lrhoe, Lphi, Urho, Urhoe) is destructured into 4 names, giving
   * Urho := Lphi = 0 and Urhoe := Urho = Inf. 0: the intended Urho = Urhoe = Inf. */
  int32_t reference_semantics;
  int32_t precision;               /* p2de_precision */
  /* SubcellLimiter's shockcapture (Solver.jl:65-74): 0 NoShockCapture, 1
   * HennemannShockCapture(a, c), whose per-element blending factor
   * (shock_capture.jl:118-137) caps every subcell factor of the element. */
  int32_t shock_capture;
  int32_t rhs_limiter;             /* p2de_rhs_limiter */
  double shock_capture_a;
  double shock_capture_c;
  double bound_beta;               /* beta of the Relaxed...CellEntropyBound types, else unused */
  int32_t approximation_basis;     /* p2de_basis */
  int32_t entropyproj_limiter;     /* p2de_entropyproj_limiter */
  int32_t equation;                /* p2de_equation */
  int32_t reserved_;               /* 0 */
} p2de_param;

/* Mesh and boundary data. geom/mapP/mapI/mapO/Ival follow StateParam.bcdata
 * (src/common/types/StateParam.jl:1-7) and GeomData (Solver.jl:185-190) for affine
 * elements. Indices are Julia's 1-based linear indices into (Nfp, K) face arrays.
 * mapW/mapS are boundary kinds that BCData does not have (used by the double Mach
 * reflection problem); pass 0 counts to leave them out. */
typedef struct p2de_mesh {
  const double* geom;    /* K x 5, element-major: J, rxJ, sxJ, ryJ, syJ */
  const int64_t* mapP;   /* Nfp*K, 1-based exterior face-node index (self on boundaries) */
  const int64_t* mapI;   /* inflow (static Dirichlet) face nodes, 1-based */
  int64_t nI;
  const double* Ival;    /* nI x 4 conservative states */
  const int64_t* mapO;   /* outflow (copy interior node) face nodes, 1-based */
  int64_t nO;
  const int64_t* mapW;   /* reflecting-wall face nodes, 1-based */
  int64_t nW;
  const int64_t* mapS;   /* moving oblique shock Dirichlet face nodes, 1-based */
  int64_t nS;
  const double* xyS;     /* nS x 2 physical coordinates of the mapS nodes */
  /* state at mapS node (x,y), time t: post if x < shock_x0 + (y + shock_speed*t)*shock_inv_slope else pre */
  double shock_x0;
  double shock_inv_slope;
  double shock_speed;
  double shock_post[4];
  double shock_pre[4];
} p2de_mesh;

/* Fields readable with p2de_get_field (state.preallocation members). Shapes are those of
 * CompressibleEulerIdealGas{Dim2}; p2de_solver_field_count gives each solver's size. KPP has
 * one double per state; CompressibleEulerIdealGas{Dim1} has SVector{3} states, SVector{1,
 * SVector{3}} flux pairs (3 doubles) and L_local (Nq+N1D) x 1 x K per stage. */
typedef enum p2de_field {
  P2DE_FIELD_UQ = 0,      /* Nq x K SVector{4} */
  P2DE_FIELD_RHSU = 1,    /* Nq x K SVector{4} */
  P2DE_FIELD_RHSL = 2,    /* Nq x K SVector{4} */
  P2DE_FIELD_RHSH = 3,    /* Nq x K SVector{4} */
  P2DE_FIELD_RHSXYL = 4,  /* Nq x K SVector{2,SVector{4}} */
  P2DE_FIELD_RHSXYH = 5,  /* Nq x K SVector{2,SVector{4}} */
  P2DE_FIELD_BF_L = 6,    /* Nfp x K SVector{2,SVector{4}} */
  P2DE_FIELD_BF_H = 7,    /* Nfp x K SVector{2,SVector{4}} */
  P2DE_FIELD_L_LOCAL = 8, /* (Nq+N1D) x 2 x K for one stage */
  P2DE_FIELD_RESW = 9,    /* Nq x K SVector{4} */
  P2DE_FIELD_L = 10,      /* K for one stage: ZhangShuLimiter's factor L[k, nstage] before the
                             shock-capture cap (zhangshu.jl:44) */
  P2DE_FIELD_THETA_LOCAL = 11, /* Nfp x K for one stage: the entropy-projection limiting factor
                                  theta_local[i, k, nstage] (1 without the limiter) */
  /* The subcell fluxes f_bar_H, f_bar_L of the limiter cache (State.jl:131-185) of the last
   * limited stage (subcell limiter, LimitedDG; accumulate_f_bar!, subcell.jl:163-206): the
   * reference's tuple of two (Nq+N1D) x K SVector{4} arrays, x then y, one after the other:
   * F[c + 4*(i + (Nq+N1D)*(k + K*d))], d = 0 (x: face si + (N1D+1) sj), 1 (y: si + N1D sj) */
  P2DE_FIELD_F_BAR_H = 12,
  P2DE_FIELD_F_BAR_L = 13
} p2de_field;

typedef struct p2de_solver p2de_solver;

/* Version of this ABI (P2DE_ABI_VERSION). */
int p2de_abi_version(void);

/* Number of doubles in a field for a solver of degree N with K elements
 * (CompressibleEulerIdealGas, Nc = 4). */
int p2de_field_count(int32_t N, int32_t K, int32_t field, int64_t* count);

/* Number of doubles in a field of this solver (its equation's Nc). */
int p2de_solver_field_count(p2de_solver* s, int32_t field, int64_t* count);

/* Replaces initialize_DG (src/dg/init.jl:44-60): builds the GLL operators for
 * degree N, uploads the mesh/BC data and allocates the device state on `device`.
 * Uq is left zero; set it with p2de_set_Uq (init_U!, init.jl:342-361). */
int p2de_initialize_DG(const p2de_param* param, const p2de_mesh* mesh, int device,
                       p2de_solver** out);

/* Releases the handle and its device memory. */
int p2de_destroy(p2de_solver* s);

/* Copies Nq*K*4 doubles from host into state.preallocation.Uq. */
int p2de_set_Uq(p2de_solver* s, const double* Uq);

/* Copies a field to the host; nstage (1..3) selects the L_local stage. */
int p2de_get_field(p2de_solver* s, int32_t field, int32_t nstage, double* out);

/* Replaces rhs!(state, solver, state_param, time_param) (src/dg/rhs/rhs.jl:5-13)
 * for the LimitedDG / LowOrderPositivity / FluxDiffRHS dispatches: computes rhsU
 * from Uq at time t with TimeParam(dt, nstage) and returns the positivity-CFL dt
 * of low_order_graph_viscosity.jl:32-40 (stage 1) or dt unchanged otherwise. */
int p2de_rhs(p2de_solver* s, double t, double dt, int32_t nstage, double* dt_out);

/* One pass of the SSP33! time loop body (src/timestepping/SSPRK33.jl:125-139):
 * advances Uq from *t by the returned dt and updates *t. */
int p2de_ssp33_step(p2de_solver* s, double* t, double* dt_out);

/* SSP33! (SSPRK33.jl:1-62) without snapshots: steps from param.t0 until t >= T.
 * Returns the final time, the step count and the last dt. */
int p2de_ssp33(p2de_solver* s, double* t_out, int64_t* steps_out, double* dt_last);

/* Runs `nsteps` SSP-RK3 steps (or stops at T) with the whole step captured in a
 * CUDA graph; t and dt stay on the device between steps. */
int p2de_ssp33_advance(p2de_solver* s, int64_t nsteps, double* t, int64_t* steps_done);

/* Device pointer of a field (for callers that keep data resident). */
int p2de_device_ptr(p2de_solver* s, int32_t field, void** dptr);

/* CUDA stream (cudaStream_t) used for every launch of this solver. */
int p2de_set_stream(p2de_solver* s, void* stream);

/* Number of kernel launches issued by this solver since creation. */
int p2de_launch_count(p2de_solver* s, int64_t* count);

/* Min density and min internal energy over all nodes of Uq (device reduction). */
int p2de_min_rho_rhoe(p2de_solver* s, double* min_rho, double* min_rhoe);

/* check_conservation (src/dg/utils.jl:1-12) on the device: totals[c] = sum over elements
 * and nodes of J wq Uq[c]; *sum = the four summed (the reference's return value). Either
 * output may be NULL. Deterministic: fixed grid and reduction order. */
int p2de_check_conservation(p2de_solver* s, double totals[4], double* sum);

/* calculate_error (src/dg/postprocess.jl:1-46) on the device against exact conservative
 * values at the nodes (host array in the layout of Uq): out = relative L1, L2, Linf
 * errors summed over the components whose exact Linf norm exceeds 1e-14. */
int p2de_calculate_error(p2de_solver* s, const double* exact_Uq, double out[3]);

/* Min density and min internal energy of each RK stage of the last step, as
 * recorded by the stage update: out[2*(stage-1)] = min rho, out[2*(stage-1)+1] = min rhoe. */
int p2de_stage_minima(p2de_solver* s, double out[6]);

/* Runs `nsteps` SSP-RK3 steps from *t with the kernels launched one by one and
 * CUDA events around each; returns the mean milliseconds per launch of stage kernel A
 * (ms[0]), stage kernel B (ms[1]) and the step-begin kernel (ms[2]). */
int p2de_profile_steps(p2de_solver* s, int64_t nsteps, double* t, double ms[3]);

/* Work counters since the last reset: out[0] = quadratic internal-energy bound
 * solves evaluated (limiter_utils.jl:108-132); the others are skipped exactly. */
int p2de_read_counters(p2de_solver* s, uint64_t out[1], int32_t reset);

/* Thread layouts. 2D solves: the layout of the high-order volume phases of stage kernel A
 * (the two-point fluxes of every node pair of a line and their gather into each node), FLAT
 * or LINES_PER_WARP. Line (1D) solves: the layout of the high-order and limiter kernel, FLAT
 * (one thread per element) or TEAM (a team of 16 lanes per element, for solves too small to
 * fill the GPU one thread per element); a Line solve starts with TEAM below 2048 elements,
 * FLAT from there. Results do not depend on the layout: every value is computed by the same
 * code in each. No counterpart in the reference (a launch parameter of this implementation). */
typedef enum p2de_layout {
  P2DE_LAYOUT_FLAT = 0,           /* flat loops over (element, pair) and (element, node) */
  P2DE_LAYOUT_LINES_PER_WARP = 1, /* whole 1D lines per warp: a warp computes the pairs of its
                                     lines, synchronizes only itself and gathers its lines'
                                     nodes (axis-aligned LGL elements; others run flat) */
  P2DE_LAYOUT_TEAM = 2            /* Line solves: a team of lanes per element */
} p2de_layout;

int p2de_set_layout(p2de_solver* s, int32_t layout);
int p2de_get_layout(p2de_solver* s, int32_t* layout);
/* Threads per block of stage kernel A: 64 or 128 (the default). Results do not depend on it. */
int p2de_set_threads_per_block(p2de_solver* s, int32_t threads);
int p2de_get_threads_per_block(p2de_solver* s, int32_t* threads);

/* Elements per thread block of the stage kernels (1..epb_max, the shared-memory limit).
 * Results do not depend on it: each element's arithmetic is the same at every value.
 * No counterpart in the reference (a launch parameter of this implementation). */
int p2de_set_elements_per_block(p2de_solver* s, int32_t epb);
int p2de_get_elements_per_block(p2de_solver* s, int32_t* epb, int32_t* epb_max);
/* Times stage kernel A at candidate elements-per-block, thread layouts and threads per block
 * (stage scratch only: the state is unchanged), keeps the fastest and returns its elements
 * per block and milliseconds; p2de_get_layout and p2de_get_threads_per_block give the rest. */
int p2de_autotune(p2de_solver* s, int32_t* best_epb, double* best_ms);

/* ---- Batches of independent solves ---------------------------------------------------
 * Many solves of uneven mesh size and degree advanced together: one persistent launch
 * per RK stage over a device work list of (solve, element range) tasks; each solve keeps
 * its own CFL step and final time. Device memory comes from one pool of pool_bytes
 * allocated at creation (the HBM budget). A solve's result is bitwise the result the
 * same solve has alone (p2de_ssp33_step): the element arithmetic is shared.
 * SSP33! (SSPRK33.jl:1-62) applied to each member. */
typedef struct p2de_batch p2de_batch;

int p2de_batch_create(int device, int32_t precision, size_t pool_bytes, int32_t max_solves, p2de_batch** out);
int p2de_batch_destroy(p2de_batch* b);
/* Device bytes one solve takes in the pool. */
int p2de_batch_solve_bytes(const p2de_param* param, int64_t nI, int64_t nS, size_t* bytes);
/* Admits a solve (copies mesh data and Uq); P2DE_ERR_BUDGET when it does not fit. */
int p2de_batch_add(p2de_batch* b, const p2de_param* param, const p2de_mesh* mesh, const double* Uq, int32_t* slot);
/* Returns the solve's memory to the pool. */
int p2de_batch_remove(p2de_batch* b, int32_t slot);
/* Advances every member by nsteps SSP-RK3 steps (members at their T stay put). */
int p2de_batch_step(p2de_batch* b, int64_t nsteps);
int p2de_batch_state(p2de_batch* b, int32_t slot, double* t, double* dt, int64_t* steps, int32_t* done,
                     int32_t* status);
/* (t, steps, done, status) of every slot, out[4*slot + ...]; status -1 for empty slots. */
int p2de_batch_states(p2de_batch* b, double* out);
int p2de_batch_get_Uq(p2de_batch* b, int32_t slot, double* Uq);
int p2de_batch_memory(p2de_batch* b, size_t* used, size_t* capacity);
int p2de_batch_launch_count(p2de_batch* b, int64_t* count);
int p2de_batch_last_error(p2de_batch* b, char* buf, size_t len);
/* Elements per block of the batch's tasks for degree N (1..5); as for one solve,
 * results do not depend on it. */
int p2de_batch_set_elements_per_block(p2de_batch* b, int32_t N, int32_t epb);
int p2de_batch_get_elements_per_block(p2de_batch* b, int32_t N, int32_t* epb, int32_t* epb_max);
/* Thread layout (p2de_layout) of the batch's tasks for degree N; results do not depend on it. */
int p2de_batch_set_layout(p2de_batch* b, int32_t N, int32_t layout);
int p2de_batch_get_layout(p2de_batch* b, int32_t N, int32_t* layout);
/* Per degree present, times batched stage kernel A over that degree's members at
 * candidate elements-per-block and thread layouts (no state changes) and keeps the
 * fastest; best_epb[N-1] receives its elements per block (0 for absent degrees) and
 * p2de_batch_get_layout its layout. */
int p2de_batch_autotune(p2de_batch* b, int32_t best_epb[5]);

/* ---- Continuous-batching server -------------------------------------------------------
 * A worker thread admits submitted solves into a batch as slots and HBM budget free up
 * (first come first served, skipping requests that do not fit yet), advances the batch
 * steps_per_tick steps at a time, and retires each solve when it reaches its T, keeping
 * its final state for p2de_server_result. Latency = retirement - submission. */
typedef struct p2de_server p2de_server;

int p2de_server_create(int device, int32_t precision, size_t hbm_budget_bytes, int32_t max_active,
                       int32_t steps_per_tick, p2de_server** out);
/* Thread-safe; copies the request's data. P2DE_ERR_BUDGET if it can never fit. */
int p2de_server_submit(p2de_server* s, const p2de_param* param, const p2de_mesh* mesh, const double* Uq,
                       int64_t* request_id);
/* state: 0 queued, 1 running, 2 done, 3 failed; latency in seconds once finished. */
int p2de_server_poll(p2de_server* s, int64_t request_id, int32_t* state, double* latency_s, double* t_final,
                     int64_t* steps);
int p2de_server_wait(p2de_server* s, int64_t request_id, double timeout_s, int32_t* state);
/* Copies a finished request's final Uq and forgets the request. */
int p2de_server_result(p2de_server* s, int64_t request_id, double* Uq);
/* completed, failed, active, queued, pool bytes in use, pool capacity, ticks, busy seconds */
int p2de_server_stats(p2de_server* s, double out[8]);
int p2de_server_destroy(p2de_server* s);

/* ---- Right-hand side without device allocation -------------------------------------
 * No counterpart in the reference. For callers that cannot call cudaMalloc when they
 * need a right-hand side: a process whose device memory is reserved up front by its own
 * pool allocator (a Julia or serving process with a fixed HBM budget, where one more
 * cudaMalloc fails or breaks the budget), or an application that allocates device memory
 * only at start-up. All scratch (subcell fluxes, blending factors, device scalars,
 * operator table) lives in one static device array of P2DE_NOALLOC_SCRATCH_BYTES that
 * every GPU loading this entry point keeps until the process exits; problems needing
 * more are rejected with P2DE_ERR_BUDGET (p2de_noalloc_max_elements gives the limit per
 * degree). The array is shared by all calls and keeps the last call's contents (the
 * operator table is rebuilt when N or ZEROTOL changes; everything else a call reads is
 * written by that call), so calls that overlap on the GPU race. The first call on a
 * device does a one-time set-up (the array's device address and kernel attributes) and
 * should come before any stream capture. Each call synchronizes `stream` before it
 * returns. Inputs and outputs are caller-owned device arrays in the layouts above. */
#define P2DE_NOALLOC_SCRATCH_BYTES (32u * 1024u * 1024u)

typedef struct p2de_device_mesh {
  const double* geom;    /* device, K x 5: J, rxJ, sxJ, ryJ, syJ */
  const int32_t* nbr;    /* device, Nfp*K: 0-based exterior face-node index (mapP - 1) */
  const int8_t* bc;      /* device, Nfp*K: 0 interior, 1 inflow, 2 outflow, 3 wall, 4 moving shock */
  const int32_t* bcidx;  /* device, Nfp*K: row of Ival (code 1) or xyS (code 4); may be NULL without those */
  const double* Ival;    /* device, nI x 4 */
  int64_t nI;
  const double* xyS;     /* device, nS x 2 */
  int64_t nS;
  double shock_x0;
  double shock_inv_slope;
  double shock_speed;
  double shock_post[4];
  double shock_pre[4];
  int32_t axis_aligned;  /* 1 if every element has sxJ = ryJ = 0 */
} p2de_device_mesh;

/* Largest K that fits the static scratch for degree N. */
int p2de_noalloc_max_elements(int32_t N, int64_t* K_max);

/* rhs! (rhs.jl:5-13) for device-resident Uq (Nq*K*4) into device rhsU, on `stream`
 * (cudaStream_t, NULL for the legacy stream), with no device allocation. Returns the
 * stage-1 positivity-CFL dt (or dt) in *dt_out, on the host. */
int p2de_rhs_noalloc(const p2de_param* param, const p2de_device_mesh* mesh, const double* Uq, double t, double dt,
                     int32_t nstage, double* rhsU, double* dt_out, void* stream);

/* Last error message of this handle (or of the last failed create when s is NULL). */
int p2de_last_error(p2de_solver* s, char* buf, size_t len);

#ifdef __cplusplus
}
#endif

#endif /* P2DE_H */
