// C ABI of libp2de_gpu.so (include/p2de.h): solver handle, device memory, the
// SSP-RK3 step sequence and its CUDA-graph replay.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstddef>
#include <cstdio>
#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/p2de.h"
#include "p2de_args.h"
#include "p2de_diag.h"
#include "p2de_launch.h"
#include "p2de_line.h"
#include "p2de_physics.cuh"
#include "p2de_stage.cuh"
#include "p2de_tables.h"

using namespace p2de;

namespace {

std::mutex g_err_mu;
std::string g_last_create_error;

// --- small kernels ------------------------------------------------------------------

// SSPRK33.jl:126 and low_order_graph_viscosity.jl:230: dt = min(CFL*dt0, T - t) is the
// stage-1 limiter dt and the initial value of the positivity-CFL minimum.
__global__ void k_step_begin(double* scal, unsigned long long* dtmin, long long* minrec, int* status, double CFL,
                             double dt0, double T) {
  if (threadIdx.x != 0) return;
  double t = scal[S_T];
  if (!(t < T) || *status != 0) {
    scal[S_DONE] = 1.0;
    return;
  }
  scal[S_DONE] = 0.0;
  double dt = jmin(CFL * dt0, T - t);
  scal[S_DT_LIM] = dt;
  if (!(dt > 0.0)) {
    atomicOr(status, ST_BAD_DT);
    scal[S_DONE] = 1.0;
    return;
  }
  *dtmin = (unsigned long long)__double_as_longlong(dt);
  long long inf_key = 0x7ff0000000000000LL;
  for (int i = 0; i < 6; ++i) minrec[i] = inf_key;
}

__device__ __forceinline__ long long okey(double x) {
  long long b = __double_as_longlong(x);
  return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}

__global__ void k_min_rho_rhoe(const double* Uq, size_t nodes, long long* out) {
  double rmin = INFINITY, emin = INFINITY;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < nodes; i += (size_t)gridDim.x * blockDim.x) {
    const double* U = Uq + 4 * i;
    double re = rhoe_ufun(U[0], U[1], U[2], U[3]);
    rmin = fmin(rmin, U[0]);
    emin = fmin(emin, re);
  }
  for (int o = 16; o > 0; o >>= 1) {
    rmin = fmin(rmin, __shfl_xor_sync(0xffffffffu, rmin, o));
    emin = fmin(emin, __shfl_xor_sync(0xffffffffu, emin, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMin(&out[0], okey(rmin));
    atomicMin(&out[1], okey(emin));
  }
}

__global__ void k_geom_table(const double* geom, int K, double* out) {
  const long long w = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (w >= (long long)K * kGeomFactors) return;
  const int k = (int)(w / kGeomFactors), q = (int)(w % kGeomFactors);
  geom_factor(geom + 5 * (size_t)k, q, out + (size_t)k * kGeomStride);
}

// initialize_s_modified! (subcell.jl:21-35) for one solve (phi_min_body, one block of 1024)
__global__ void __launch_bounds__(1024) k_phi_min(const double* Uq, size_t nodes, double gamma, const double* scal,
                                                  double t0, double* out) {
  phi_min_body(Uq, nodes, gamma, scal, t0, out);
}

double key_to_double(long long k) {
  long long b = k ^ ((k >> 63) & 0x7fffffffffffffffLL);
  double d;
  std::memcpy(&d, &b, 8);
  return d;
}

// --- operator tables per device -------------------------------------------------------

// The tables depend on the degree, the basis and ZEROTOL (build_op_table drops entries at
// or below it), so each device keeps one set per ZEROTOL value in use, until exit.
struct DeviceTables {
  uint64_t zerotol_bits = 0;
  OpTable* d_tables = nullptr;  // LGL N1D = 2..6, then Gauss N1D = 2..6
};
std::mutex g_tab_mu;
std::vector<DeviceTables> g_tabs[64];

cudaError_t device_tables(int dev, double zerotol, OpTable** out) {
  std::lock_guard<std::mutex> lk(g_tab_mu);
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  uint64_t bits;
  std::memcpy(&bits, &zerotol, sizeof bits);
  for (const DeviceTables& t : g_tabs[dev])
    if (t.zerotol_bits == bits) {
      *out = t.d_tables;
      return cudaSuccess;
    }
  // LGL tables for N1D = 2..6, then the Gauss tables in the same order
  std::vector<OpTable> h(2 * (kMaxN1D - 1));
  for (int N = 1; N < kMaxN1D; ++N) {
    build_op_table(N, zerotol, &h[N - 1], 0);
    build_op_table(N, zerotol, &h[kMaxN1D - 1 + N - 1], 1);
  }
  DeviceTables t;
  t.zerotol_bits = bits;
  cudaError_t e = cudaMalloc(&t.d_tables, sizeof(OpTable) * h.size());
  if (e != cudaSuccess) return e;
  e = cudaMemcpy(t.d_tables, h.data(), sizeof(OpTable) * h.size(), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(t.d_tables);
    return e;
  }
  g_tabs[dev].push_back(t);
  *out = t.d_tables;
  return cudaSuccess;
}

cudaError_t prepare_n1d(int n1d, StageGeometry* geo) {
  switch (n1d) {
    case 2: return stage_prepare<2>(geo);
    case 3: return stage_prepare<3>(geo);
    case 4: return stage_prepare<4>(geo);
    case 5: return stage_prepare<5>(geo);
    case 6: return stage_prepare<6>(geo);
  }
  return cudaErrorInvalidValue;
}
cudaError_t launch_a_one(int n1d, const StageArgs& a, bool mixed, cudaStream_t st) {
  switch (n1d) {
    case 2: return launch_stage_a<2>(a, mixed, st);
    case 3: return launch_stage_a<3>(a, mixed, st);
    case 4: return launch_stage_a<4>(a, mixed, st);
    case 5: return launch_stage_a<5>(a, mixed, st);
    case 6: return launch_stage_a<6>(a, mixed, st);
  }
  return cudaErrorInvalidValue;
}
// kernel A. The TVD bounds need every element's low-order density: a first launch stops
// after the low-order RHS and stores them, then the full launch reads its stencils. The
// relaxed min-entropy bounds need the initial state's minimum of phi: at stage 1 a
// one-block reduction runs first (it returns at once unless t == t0).
bool needs_phi_min(const StageArgs& a) {
  return (a.flags & F_MIN_ENTROPY) && (a.flags & F_RELAXED) && a.nstage == 1;
}
// Gauss collocation with a cell-entropy bound: the interface step between kernels A and B
bool needs_es_interface(const StageArgs& a) { return (a.flags & F_GAUSS) && (a.flags & F_CELL_ENTROPY); }
int a_launches(const StageArgs& a) {
  return ((a.flags & F_TVD) ? 2 : 1) + (needs_phi_min(a) ? 1 : 0) + ((a.flags & F_GAUSS) ? 1 : 0) +
         (needs_es_interface(a) ? 1 : 0);
}
cudaError_t launch_es_interface_n1d(int n1d, const StageArgs& a, cudaStream_t st) {
  switch (n1d) {
    case 2: return launch_es_interface<2>(a, st);
    case 3: return launch_es_interface<3>(a, st);
    case 4: return launch_es_interface<4>(a, st);
    case 5: return launch_es_interface<5>(a, st);
    case 6: return launch_es_interface<6>(a, st);
  }
  return cudaErrorInvalidValue;
}
cudaError_t launch_gauss_proj_n1d(int n1d, const StageArgs& a, cudaStream_t st) {
  switch (n1d) {
    case 2: return launch_gauss_proj<2>(a, st);
    case 3: return launch_gauss_proj<3>(a, st);
    case 4: return launch_gauss_proj<4>(a, st);
    case 5: return launch_gauss_proj<5>(a, st);
    case 6: return launch_gauss_proj<6>(a, st);
  }
  return cudaErrorInvalidValue;
}
// Gauss collocation: the face projection of the stage first (every element's projected
// face states must exist before kernel A reads its neighbours')
cudaError_t launch_a_n1d(int n1d, const StageArgs& a, bool mixed, cudaStream_t st) {
  if (a.flags & F_GAUSS) {
    cudaError_t e = launch_gauss_proj_n1d(n1d, a, st);
    if (e != cudaSuccess) return e;
  }
  if (needs_phi_min(a)) {
    k_phi_min<<<1, 1024, 0, st>>>(a.Uq, (size_t)a.K * n1d * n1d, a.gamma, a.scal, a.t0, a.phimin);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  if (a.flags & F_TVD) {
    StageArgs lo = a;
    lo.flags = (a.flags | F_LOW_ONLY) & ~(F_CFL | F_WRITE_DEBUG);
    cudaError_t e = launch_a_one(n1d, lo, mixed, st);
    if (e != cudaSuccess) return e;
  }
  cudaError_t e = launch_a_one(n1d, a, mixed, st);
  if (e != cudaSuccess || !needs_es_interface(a)) return e;
  return launch_es_interface_n1d(n1d, a, st);
}
cudaError_t launch_b_n1d(int n1d, const StageArgs& a, cudaStream_t st) {
  switch (n1d) {
    case 2: return launch_stage_b<2>(a, st);
    case 3: return launch_stage_b<3>(a, st);
    case 4: return launch_stage_b<4>(a, st);
    case 5: return launch_stage_b<5>(a, st);
    case 6: return launch_stage_b<6>(a, st);
  }
  return cudaErrorInvalidValue;
}

}  // namespace

namespace p2de {
cudaError_t launch_geom_table(const double* geom, int K, double* out, cudaStream_t st) {
  const long long items = (long long)K * kGeomFactors;
  k_geom_table<<<(int)((items + 255) / 256), 256, 0, st>>>(geom, K, out);
  return cudaGetLastError();
}
}  // namespace p2de

struct p2de_solver {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  p2de_param prm{};
  int N = 0, N1D = 0, Nq = 0, Nfp = 0, K = 0, NSF = 0;
  StageGeometry geo{};
  bool mixed = false;
  bool axis_aligned = true;
  // device memory
  double *Uq = nullptr, *resW = nullptr, *rhsL = nullptr, *rhsH = nullptr, *rhsU = nullptr;
  double *rhsxyL = nullptr, *rhsxyH = nullptr, *BFL = nullptr, *BFH = nullptr;
  double *fbar = nullptr, *Lpre = nullptr, *Lfin = nullptr, *geom = nullptr, *Ival = nullptr, *xyS = nullptr;
  double* geomx = nullptr;  // K x 16 geometry factors
  double* scal = nullptr;
  int32_t *nbr = nullptr, *bcidx = nullptr;
  int8_t* bc = nullptr;
  unsigned long long* dtmin = nullptr;
  long long* minrec = nullptr;
  long long* minbuf = nullptr;
  int* status = nullptr;
  unsigned long long* counters = nullptr;
  OpTable* ops = nullptr;
  double *diag_partial = nullptr, *diag_out = nullptr, *exact = nullptr;  // diagnostics, on first use
  double* rhoL = nullptr;                                                  // TVD bounds only
  double* Lelem = nullptr;                                                 // 3 x K ZhangShuLimiter factors
  double* phimin = nullptr;                                                // initial min of phi
  bool gauss = false;                                                      // GaussCollocation
  bool kpp = false;                                                        // KPP{Dim2}: Nc = 1
  double *ufproj = nullptr, *theta = nullptr;                              // Gauss face projection
  LineSolve* line = nullptr;                                               // CompressibleEulerIdealGas{Dim1}
  int diag_nblocks = 0;
  StageArgs base{};
  int64_t launches = 0;
  double line_dt = 0.0;  // last dt of the Line path
  cudaGraphExec_t graph = nullptr;
  std::string err;
  std::vector<void*> allocs;
};

namespace {

int fail(p2de_solver* s, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (s)
    s->err = buf;
  else {
    std::lock_guard<std::mutex> lk(g_err_mu);
    g_last_create_error = buf;
  }
  return code;
}

#define CK(call)                                                                                   \
  do {                                                                                             \
    cudaError_t e_ = (call);                                                                       \
    if (e_ != cudaSuccess) return fail(s, P2DE_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

template <typename T>
cudaError_t dalloc(p2de_solver* s, T** p, size_t count) {
  void* q = nullptr;
  size_t bytes = sizeof(T) * (count > 0 ? count : 1);
  cudaError_t e = cudaMalloc(&q, bytes);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(q, 0, bytes, s->stream);
  if (e != cudaSuccess) return e;
  s->allocs.push_back(q);
  *p = (T*)q;
  return cudaSuccess;
}

// the operator table of the solve: LGL tables for N1D = 2..6, then the Gauss tables
const OpTable* table_of(const p2de_solver* s) {
  return s->ops + (s->N1D - 2) + (s->gauss ? kMaxN1D - 1 : 0);
}

int flags_for(const p2de_solver* s, int nstage, bool update, bool debug) {
  int f = 0;
  switch (s->prm.rhs_type) {
    case P2DE_RHS_LOW_ORDER_POSITIVITY: f |= F_DO_LOW | F_RHSU_FROM_L; break;
    case P2DE_RHS_ENTROPY_STABLE: f |= F_DO_HIGH | F_RHSU_FROM_H; break;
    default: f |= F_DO_LOW | F_DO_HIGH | F_DO_LIMIT; break;
  }
  if ((f & F_DO_LOW) && nstage == 1) f |= F_CFL;
  if (s->axis_aligned) f |= F_AXIS_ALIGNED;
  if (f & F_DO_LIMIT) {
    if (s->prm.rhs_limiter == P2DE_LIMITER_ZHANG_SHU) {
      f = (f & ~F_DO_LIMIT) | F_ZHANG_SHU;  // the bound type is not read
    } else {
      const int b = s->prm.bound_type;
      f |= bound_flags(b);
      // the min-entropy bounds read their 5-tuple with 5 names (limiter_utils.jl:19-24)
      if (s->prm.reference_semantics && !(f & F_MIN_ENTROPY)) f |= F_REF_SEM;
    }
  }
  if (s->prm.precision == P2DE_PRECISION_MIXED_ACC64) f |= F_ACC64;
  if (s->prm.shock_capture == 1 && (f & (F_DO_LIMIT | F_ZHANG_SHU))) f |= F_SHOCK;
  if (s->kpp) f |= F_KPP;
  if (s->prm.low_order_surface_flux == P2DE_FLUX_LAX_FRIEDRICHS_ON_PROJECTED_VAL) f |= F_LFPROJ;
  if (s->gauss) {
    f |= F_GAUSS;
    if (s->prm.entropyproj_limiter == P2DE_ENTROPYPROJ_NODEWISE_SCALED_EXTRAPOLATION) f |= F_EPROJ;
  }
  if (update) f |= F_UPDATE;
  if (debug) f |= F_WRITE_DEBUG;
  return f;
}

int check_status(p2de_solver* s) {
  int st = 0;
  CK(cudaMemcpyAsync(&st, s->status, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  if (st & (ST_NOT_POSITIVE | ST_NAN)) return fail(s, P2DE_ERR_NOT_POSITIVE, "density or internal energy not positive (status %d)", st);
  if (st & ST_BAD_DT) return fail(s, P2DE_ERR_BAD_DT, "time step not positive (status %d)", st);
  return P2DE_OK;
}

// Issues the 7 launches of one SSP-RK3 step on s->stream.
int enqueue_step(p2de_solver* s) {
  k_step_begin<<<1, 32, 0, s->stream>>>(s->scal, s->dtmin, s->minrec, s->status, s->prm.CFL, s->prm.dt0, s->prm.T);
  CK(cudaGetLastError());
  s->launches += 1;
  for (int stage = 1; stage <= 3; ++stage) {
    StageArgs a = s->base;
    a.nstage = stage;
    a.flags = flags_for(s, stage, true, false);
    CK(launch_a_n1d(s->N1D, a, s->mixed, s->stream));
    CK(launch_b_n1d(s->N1D, a, s->stream));
    s->launches += a_launches(a) + 1;
  }
  return P2DE_OK;
}

// launches of one step: the step begin, then per stage kernel A (twice for TVD bounds), B
int step_launches(const p2de_solver* s) {
  int n = 1;
  for (int stage = 1; stage <= 3; ++stage) {
    StageArgs a = s->base;
    a.nstage = stage;
    a.flags = flags_for(s, stage, true, false);
    n += a_launches(a) + 1;
  }
  return n;
}

void free_all(p2de_solver* s) {
  if (s->line) line_destroy(s->line);
  s->line = nullptr;
  if (s->graph) cudaGraphExecDestroy(s->graph);
  for (void* p : s->allocs) cudaFree(p);
  s->allocs.clear();
  if (s->own_stream && s->stream) cudaStreamDestroy(s->stream);
}

// CompressibleEulerIdealGas{Dim1}: the handle's common fields point at the Line state, so
// the diagnostics (min rho/rhoe, conservation, errors, stage minima) serve both
int create_line(const p2de_param* prm, const p2de_mesh* mesh, int device, p2de_solver** out) {
  {
    std::string err;
    const int rc = line_validate(prm, mesh, err);
    if (rc != P2DE_OK) return fail(nullptr, rc, "%s", err.c_str());
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(nullptr, P2DE_ERR_NO_DEVICE, "no CUDA device");
  if (device < 0 || device >= ndev) return fail(nullptr, P2DE_ERR_INVALID_ARGUMENT, "device %d of %d", device, ndev);
  auto* s = new p2de_solver();
  s->device = device;
  s->prm = *prm;
  s->N = prm->N;
  s->N1D = prm->N + 1;
  s->Nq = s->N1D;
  s->Nfp = 2;
  s->K = prm->K;
  s->gauss = prm->approximation_basis == P2DE_BASIS_GAUSS;
  auto bail = [&](int code) {
    {
      std::lock_guard<std::mutex> lk(g_err_mu);
      g_last_create_error = s->err;
    }
    free_all(s);
    delete s;
    return code;
  };
  if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) {
    fail(s, P2DE_ERR_CUDA, "device setup failed");
    return bail(P2DE_ERR_CUDA);
  }
  s->own_stream = true;
  std::string err;
  const int rc = line_create(prm, mesh, s->stream, &s->line, err);
  if (rc != P2DE_OK) {
    s->err = err;
    return bail(rc);
  }
  if (dalloc(s, &s->minbuf, 2) != cudaSuccess || dalloc(s, &s->counters, 8) != cudaSuccess) {
    fail(s, P2DE_ERR_OUT_OF_MEMORY, "cudaMalloc");
    return bail(P2DE_ERR_OUT_OF_MEMORY);
  }
  s->Uq = s->line->Uq;
  s->resW = s->line->resW;
  s->rhsL = s->line->rhsL;
  s->rhsH = s->line->rhsH;
  s->rhsU = s->line->rhsU;
  s->geom = s->line->geom;
  s->minrec = s->line->minrec;
  s->status = s->line->status;
  *out = s;
  return P2DE_OK;
}

int line_status(p2de_solver* s, int rc, const std::string& err) {
  if (rc != P2DE_OK) s->err = err;
  return rc;
}

}  // namespace

extern "C" {

int p2de_abi_version(void) { return P2DE_ABI_VERSION; }

int p2de_field_count(int32_t N, int32_t K, int32_t field, int64_t* count) {
  if (!count || N < 1 || N > 5 || K < 1) return P2DE_ERR_INVALID_ARGUMENT;
  int64_t n = N + 1, Nq = n * n, Nfp = 4 * n;
  switch (field) {
    case P2DE_FIELD_UQ:
    case P2DE_FIELD_RHSU:
    case P2DE_FIELD_RHSL:
    case P2DE_FIELD_RHSH:
    case P2DE_FIELD_RESW: *count = 4 * Nq * K; break;
    case P2DE_FIELD_RHSXYL:
    case P2DE_FIELD_RHSXYH: *count = 8 * Nq * K; break;
    case P2DE_FIELD_BF_L:
    case P2DE_FIELD_BF_H: *count = 8 * Nfp * K; break;
    case P2DE_FIELD_L_LOCAL: *count = (Nq + n) * 2 * K; break;
    case P2DE_FIELD_L: *count = K; break;
    case P2DE_FIELD_THETA_LOCAL: *count = Nfp * K; break;
    case P2DE_FIELD_F_BAR_H:
    case P2DE_FIELD_F_BAR_L: *count = 4 * (Nq + n) * 2 * K; break;
    default: return P2DE_ERR_INVALID_ARGUMENT;
  }
  return P2DE_OK;
}

int p2de_initialize_DG(const p2de_param* prm, const p2de_mesh* mesh, int device, p2de_solver** out) {
  p2de_solver* s = nullptr;
  if (!prm || !mesh || !out) return fail(nullptr, P2DE_ERR_INVALID_ARGUMENT, "null argument");
  *out = nullptr;
  if (prm->N < 1 || prm->N > 5) return fail(nullptr, P2DE_ERR_INVALID_ARGUMENT, "N=%d outside 1..5", prm->N);
  if (prm->K < 1) return fail(nullptr, P2DE_ERR_INVALID_ARGUMENT, "K=%d", prm->K);
  if (!mesh->geom || !mesh->mapP) return fail(nullptr, P2DE_ERR_INVALID_ARGUMENT, "geom and mapP are required");
  if (prm->equation == P2DE_EQUATION_COMPRESSIBLE_EULER_1D) return create_line(prm, mesh, device, out);
  if ((prm->low_order_surface_flux != P2DE_FLUX_LAX_FRIEDRICHS_ON_NODAL_VAL &&
       prm->low_order_surface_flux != P2DE_FLUX_LAX_FRIEDRICHS_ON_PROJECTED_VAL) ||
      prm->high_order_surface_flux != P2DE_FLUX_LAX_FRIEDRICHS_ON_PROJECTED_VAL)
    return fail(nullptr, P2DE_ERR_UNSUPPORTED,
                "surface fluxes: LaxFriedrichsOnNodalVal or LaxFriedrichsOnProjectedVal (low order), "
                "LaxFriedrichsOnProjectedVal (high order)");
  if (prm->equation < 0 || prm->equation > 2)
    return fail(nullptr, P2DE_ERR_INVALID_ARGUMENT, "equation %d out of range", prm->equation);
  if (prm->equation == P2DE_EQUATION_KPP &&
      (prm->approximation_basis != P2DE_BASIS_LOBATTO || prm->precision != P2DE_PRECISION_FP64 || mesh->nI ||
       mesh->nO || mesh->nW || mesh->nS ||
       (prm->rhs_limiter == P2DE_LIMITER_SUBCELL && prm->bound_type != P2DE_BOUND_POSITIVITY)))
    return fail(nullptr, P2DE_ERR_UNSUPPORTED,
                "KPP: LGL nodes, FP64, periodic or self-connected faces, PositivityBound or ZhangShuLimiter");
  if (prm->rhs_type < 0 || prm->rhs_type > 2 || prm->bound_type < 0 || prm->bound_type > 9 || prm->precision < 0 ||
      prm->precision > 2 || prm->shock_capture < 0 || prm->shock_capture > 1 || prm->rhs_limiter < 0 ||
      prm->rhs_limiter > 1)
    return fail(nullptr, P2DE_ERR_INVALID_ARGUMENT, "rhs_type/bound_type/precision/rhs_limiter out of range");
  if (prm->approximation_basis < 0 || prm->approximation_basis > 1 || prm->entropyproj_limiter < 0 ||
      prm->entropyproj_limiter > 1)
    return fail(nullptr, P2DE_ERR_INVALID_ARGUMENT, "approximation_basis/entropyproj_limiter out of range");
  if (prm->approximation_basis == P2DE_BASIS_GAUSS) {
    if (prm->precision != P2DE_PRECISION_FP64)
      return fail(nullptr, P2DE_ERR_UNSUPPORTED, "GaussCollocation runs in FP64 only");
  }
  const int64_t n1 = prm->N + 1, Nfp = 4 * n1, Nq = n1 * n1;
  const int64_t nfk = Nfp * prm->K;
  // validate indices before anything reaches the device
  for (int64_t i = 0; i < nfk; ++i)
    if (mesh->mapP[i] < 1 || mesh->mapP[i] > nfk)
      return fail(nullptr, P2DE_ERR_INVALID_ARGUMENT, "mapP[%lld]=%lld out of 1..%lld", (long long)i,
                  (long long)mesh->mapP[i], (long long)nfk);
  auto check_list = [&](const int64_t* m, int64_t cnt, const char* name) -> int {
    if (cnt < 0 || (cnt > 0 && !m)) return fail(nullptr, P2DE_ERR_INVALID_ARGUMENT, "%s: bad list", name);
    for (int64_t i = 0; i < cnt; ++i)
      if (m[i] < 1 || m[i] > nfk)
        return fail(nullptr, P2DE_ERR_INVALID_ARGUMENT, "%s[%lld]=%lld out of range", name, (long long)i, (long long)m[i]);
    return P2DE_OK;
  };
  int rc;
  if ((rc = check_list(mesh->mapI, mesh->nI, "mapI")) != P2DE_OK) return rc;
  if ((rc = check_list(mesh->mapO, mesh->nO, "mapO")) != P2DE_OK) return rc;
  if ((rc = check_list(mesh->mapW, mesh->nW, "mapW")) != P2DE_OK) return rc;
  if ((rc = check_list(mesh->mapS, mesh->nS, "mapS")) != P2DE_OK) return rc;
  if (mesh->nI > 0 && !mesh->Ival) return fail(nullptr, P2DE_ERR_INVALID_ARGUMENT, "Ival missing");
  if (mesh->nS > 0 && !mesh->xyS) return fail(nullptr, P2DE_ERR_INVALID_ARGUMENT, "xyS missing");
  for (int64_t k = 0; k < prm->K; ++k)
    if (!(mesh->geom[5 * k] > 0.0))
      return fail(nullptr, P2DE_ERR_INVALID_ARGUMENT, "J[%lld] = %g is not positive", (long long)k, mesh->geom[5 * k]);
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(nullptr, P2DE_ERR_NO_DEVICE, "no CUDA device");
  if (device < 0 || device >= ndev) return fail(nullptr, P2DE_ERR_INVALID_ARGUMENT, "device %d of %d", device, ndev);

  s = new p2de_solver();
  s->device = device;
  s->prm = *prm;
  s->N = prm->N;
  s->N1D = (int)n1;
  s->Nq = (int)Nq;
  s->Nfp = (int)Nfp;
  s->K = prm->K;
  s->mixed = prm->precision != P2DE_PRECISION_FP64;
  auto bail = [&](int code) {
    {
      std::lock_guard<std::mutex> lk(g_err_mu);
      g_last_create_error = s->err;
    }
    free_all(s);
    delete s;
    return code;
  };
  if (cudaSetDevice(device) != cudaSuccess) {
    fail(s, P2DE_ERR_CUDA, "cudaSetDevice failed");
    return bail(P2DE_ERR_CUDA);
  }
  if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) {
    fail(s, P2DE_ERR_CUDA, "stream create failed");
    return bail(P2DE_ERR_CUDA);
  }
  s->own_stream = true;
  cudaError_t e = prepare_n1d(s->N1D, &s->geo);
  if (e == cudaSuccess) e = device_tables(device, prm->ZEROTOL, &s->ops);
  if (e != cudaSuccess) {
    fail(s, P2DE_ERR_CUDA, "setup: %s", cudaGetErrorString(e));
    return bail(P2DE_ERR_CUDA);
  }
  s->NSF = s->geo.nsf;
  s->gauss = prm->approximation_basis == P2DE_BASIS_GAUSS;
  s->kpp = prm->equation == P2DE_EQUATION_KPP;
  if (s->gauss) {  // kernel A's Gauss layout is larger: its own elements per block
    s->geo.elems_per_block = s->geo.elems_per_block_gauss;
    s->geo.elems_per_block_max = s->geo.elems_per_block_max_gauss;
  }
  const size_t K = (size_t)s->K;
  // host-side preprocessing: neighbour indices, boundary codes, axis alignment
  std::vector<int32_t> nbr(nfk), bcidx(nfk, 0);
  std::vector<int8_t> bc(nfk, BC_INTERIOR);
  for (int64_t i = 0; i < nfk; ++i) nbr[i] = (int32_t)(mesh->mapP[i] - 1);
  for (int64_t i = 0; i < mesh->nI; ++i) {
    bc[mesh->mapI[i] - 1] = BC_INFLOW;
    bcidx[mesh->mapI[i] - 1] = (int32_t)i;
  }
  for (int64_t i = 0; i < mesh->nO; ++i) bc[mesh->mapO[i] - 1] = BC_OUTFLOW;
  for (int64_t i = 0; i < mesh->nW; ++i) bc[mesh->mapW[i] - 1] = BC_WALL;
  for (int64_t i = 0; i < mesh->nS; ++i) {
    bc[mesh->mapS[i] - 1] = BC_SHOCK;
    bcidx[mesh->mapS[i] - 1] = (int32_t)i;
  }
  s->axis_aligned = true;
  for (size_t k = 0; k < K; ++k) {
    const double* g = mesh->geom + 5 * k;
    if (g[2] != 0.0 || g[3] != 0.0) s->axis_aligned = false;
    if (!(g[0] > 0.0)) {
      fail(s, P2DE_ERR_INVALID_ARGUMENT, "J[%zu] = %g is not positive", k, g[0]);
      return bail(P2DE_ERR_INVALID_ARGUMENT);
    }
  }
#define DA(ptr, cnt)                                                                     \
  do {                                                                                   \
    cudaError_t ee = dalloc(s, &(ptr), (cnt));                                           \
    if (ee != cudaSuccess) {                                                             \
      fail(s, P2DE_ERR_OUT_OF_MEMORY, "cudaMalloc %s: %s", #ptr, cudaGetErrorString(ee)); \
      return bail(P2DE_ERR_OUT_OF_MEMORY);                                               \
    }                                                                                    \
  } while (0)
  DA(s->Uq, 4 * Nq * K);
  DA(s->resW, 4 * Nq * K);
  DA(s->rhsL, 4 * Nq * K);
  DA(s->rhsH, 4 * Nq * K);
  DA(s->rhsU, 4 * Nq * K);
  DA(s->rhsxyL, 8 * Nq * K);
  DA(s->rhsxyH, 8 * Nq * K);
  DA(s->BFL, 8 * Nfp * K);
  DA(s->BFH, 8 * Nfp * K);
  DA(s->fbar, (size_t)s->geo.fbar_per_elem * K);
  DA(s->Lpre, (size_t)2 * s->NSF * K);
  DA(s->Lfin, (size_t)3 * 2 * s->NSF * K);
  DA(s->geom, 5 * K);
  DA(s->geomx, (size_t)kGeomStride * K);
  DA(s->Ival, (size_t)4 * (mesh->nI > 0 ? mesh->nI : 1));
  DA(s->xyS, (size_t)2 * (mesh->nS > 0 ? mesh->nS : 1));
  DA(s->scal, (size_t)S_NSCAL);
  DA(s->nbr, (size_t)nfk);
  DA(s->bcidx, (size_t)nfk);
  DA(s->bc, (size_t)nfk);
  DA(s->dtmin, 1);
  DA(s->minrec, 6);
  DA(s->minbuf, 2);
  DA(s->status, 1);
  DA(s->counters, 8);
  DA(s->Lelem, (size_t)3 * K);
  DA(s->phimin, 1);
#undef DA
  auto up = [&](void* dst, const void* src, size_t bytes) {
    return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s->stream);
  };
  e = up(s->geom, mesh->geom, sizeof(double) * 5 * K);
  if (e == cudaSuccess) e = launch_geom_table(s->geom, (int)K, s->geomx, s->stream);
  if (e == cudaSuccess) e = up(s->nbr, nbr.data(), sizeof(int32_t) * nfk);
  if (e == cudaSuccess) e = up(s->bcidx, bcidx.data(), sizeof(int32_t) * nfk);
  if (e == cudaSuccess) e = up(s->bc, bc.data(), nfk);
  if (e == cudaSuccess && mesh->nI > 0) e = up(s->Ival, mesh->Ival, sizeof(double) * 4 * mesh->nI);
  if (e == cudaSuccess && mesh->nS > 0) e = up(s->xyS, mesh->xyS, sizeof(double) * 2 * mesh->nS);
  double sc[S_NSCAL] = {0};
  sc[S_T] = prm->t0;
  if (e == cudaSuccess) e = up(s->scal, sc, sizeof sc);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  if (e != cudaSuccess) {
    fail(s, P2DE_ERR_CUDA, "upload: %s", cudaGetErrorString(e));
    return bail(P2DE_ERR_CUDA);
  }
  StageArgs& a = s->base;
  a.K = s->K;
  a.epb = s->geo.elems_per_block;
  a.ops = table_of(s);
  a.Uq = s->Uq;
  a.resW = s->resW;
  a.geom = s->geom;
  a.geomx = s->geomx;
  a.nbr = s->nbr;
  a.bc = s->bc;
  a.bcidx = s->bcidx;
  a.Ival = s->Ival;
  a.xyS = s->xyS;
  a.shock_x0 = mesh->shock_x0;
  a.shock_inv_slope = mesh->shock_inv_slope;
  a.shock_speed = mesh->shock_speed;
  for (int c = 0; c < 4; ++c) {
    a.shock_post[c] = mesh->shock_post[c];
    a.shock_pre[c] = mesh->shock_pre[c];
  }
  a.gamma = prm->gamma;
  a.gm1 = prm->gamma - 1.0;
  a.CFL = prm->CFL;
  a.dt0 = prm->dt0;
  a.T = prm->T;
  a.zeta = prm->zeta;
  a.ZEROTOL = prm->ZEROTOL;
  a.rhsL = s->rhsL;
  a.rhsH = s->rhsH;
  a.rhsU = s->rhsU;
  a.rhsxyL = s->rhsxyL;
  a.rhsxyH = s->rhsxyH;
  a.BFL = s->BFL;
  a.BFH = s->BFH;
  a.fbar = s->fbar;
  a.Lpre = s->Lpre;
  a.Lfin = s->Lfin;
  a.scal = s->scal;
  a.dtmin_bits = s->dtmin;
  a.minrec = s->minrec;
  a.status = s->status;
  a.counters = s->counters;
  set_shock_capture(a, prm->N, prm->shock_capture_a, prm->shock_capture_c);
  set_bound_constants(a, prm->N, prm->t0, prm->POSTOL, prm->bound_beta);
  a.Lelem = s->Lelem;
  a.phimin = s->phimin;
  a.eta = prm->eta;
  if (s->gauss) {
    if (dalloc(s, &s->ufproj, (size_t)4 * Nfp * prm->K) != cudaSuccess ||
        dalloc(s, &s->theta, (size_t)3 * Nfp * prm->K) != cudaSuccess)
      return bail(P2DE_ERR_OUT_OF_MEMORY);
    a.ufproj = s->ufproj;
    a.theta = s->theta;
  }
  if (bound_flags(prm->bound_type) & F_TVD) {
    if (dalloc(s, &s->rhoL, (size_t)Nq * prm->K) != cudaSuccess) return bail(P2DE_ERR_OUT_OF_MEMORY);
    a.rhoL = s->rhoL;
  }
  *out = s;
  return P2DE_OK;
}

int p2de_destroy(p2de_solver* s) {
  if (!s) return P2DE_OK;
  cudaSetDevice(s->device);
  if (s->stream) cudaStreamSynchronize(s->stream);
  free_all(s);
  delete s;
  return P2DE_OK;
}

int p2de_set_Uq(p2de_solver* s, const double* Uq) {
  if (!s || !Uq) return P2DE_ERR_INVALID_ARGUMENT;
  CK(cudaSetDevice(s->device));
  if (s->line) {
    std::string err;
    return line_status(s, line_set_Uq(s->line, Uq, err), err);
  }
  const size_t nodes = (size_t)s->Nq * s->K;
  if (s->kpp) {  // one component per node, held as the first of four (the rest 0)
    std::vector<double> full(4 * nodes, 0.0);
    for (size_t i = 0; i < nodes; ++i) full[4 * i] = Uq[i];
    CK(cudaMemcpyAsync(s->Uq, full.data(), sizeof(double) * full.size(), cudaMemcpyHostToDevice, s->stream));
    CK(cudaMemsetAsync(s->status, 0, sizeof(int), s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return P2DE_OK;
  }
  CK(cudaMemcpyAsync(s->Uq, Uq, sizeof(double) * 4 * nodes, cudaMemcpyHostToDevice, s->stream));
  CK(cudaMemsetAsync(s->status, 0, sizeof(int), s->stream));
  CK(cudaStreamSynchronize(s->stream));
  return P2DE_OK;
}

int p2de_get_field(p2de_solver* s, int32_t field, int32_t nstage, double* out) {
  if (!s || !out) return P2DE_ERR_INVALID_ARGUMENT;
  if (s->line) {
    CK(cudaSetDevice(s->device));
    std::string err;
    return line_status(s, line_get_field(s->line, field, nstage, out, err), err);
  }
  int64_t cnt = 0;
  if (p2de_field_count(s->N, s->K, field, &cnt) != P2DE_OK) return fail(s, P2DE_ERR_INVALID_ARGUMENT, "bad field %d", field);
  const double* src = nullptr;
  switch (field) {
    case P2DE_FIELD_UQ: src = s->Uq; break;
    case P2DE_FIELD_RHSU: src = s->rhsU; break;
    case P2DE_FIELD_RHSL: src = s->rhsL; break;
    case P2DE_FIELD_RHSH: src = s->rhsH; break;
    case P2DE_FIELD_RHSXYL: src = s->rhsxyL; break;
    case P2DE_FIELD_RHSXYH: src = s->rhsxyH; break;
    case P2DE_FIELD_BF_L: src = s->BFL; break;
    case P2DE_FIELD_BF_H: src = s->BFH; break;
    case P2DE_FIELD_RESW: src = s->resW; break;
    case P2DE_FIELD_L_LOCAL:
      if (nstage < 1 || nstage > 3) return fail(s, P2DE_ERR_INVALID_ARGUMENT, "nstage %d", nstage);
      src = s->Lfin + (size_t)(nstage - 1) * cnt;
      break;
    case P2DE_FIELD_L:
      if (nstage < 1 || nstage > 3) return fail(s, P2DE_ERR_INVALID_ARGUMENT, "nstage %d", nstage);
      src = s->Lelem + (size_t)(nstage - 1) * cnt;
      break;
    case P2DE_FIELD_THETA_LOCAL:
      if (nstage < 1 || nstage > 3) return fail(s, P2DE_ERR_INVALID_ARGUMENT, "nstage %d", nstage);
      if (!s->gauss) {  // theta_local = 1 (clear_entropyproj_limiting_parameter_cache!)
        for (int64_t i = 0; i < cnt; ++i) out[i] = 1.0;
        return P2DE_OK;
      }
      src = s->theta + (size_t)(nstage - 1) * cnt;
      break;
    case P2DE_FIELD_F_BAR_H:
    case P2DE_FIELD_F_BAR_L: {
      // device layout per element [d][H/L][face][c] (stage kernel A, P12) -> the
      // reference's f_bar[d][face, k]
      CK(cudaSetDevice(s->device));
      const size_t nsf = (size_t)s->N1D * (s->N1D + 1), K = (size_t)s->K;
      std::vector<double> fb(16 * nsf * K);
      CK(cudaMemcpyAsync(fb.data(), s->fbar, sizeof(double) * fb.size(), cudaMemcpyDeviceToHost, s->stream));
      CK(cudaStreamSynchronize(s->stream));
      const int hl = field == P2DE_FIELD_F_BAR_H ? 0 : 1;
      const int nc = s->kpp ? 1 : 4;  // KPP: the scalar in component 0
      for (size_t d = 0; d < 2; ++d)
        for (size_t k = 0; k < K; ++k)
          for (size_t f = 0; f < nsf; ++f)
            for (int c = 0; c < nc; ++c)
              out[nc * (f + nsf * (k + K * d)) + c] = fb[16 * nsf * k + ((d * 2 + hl) * nsf + f) * 4 + c];
      return P2DE_OK;
    }
  }
  CK(cudaSetDevice(s->device));
  const bool state4 = field == P2DE_FIELD_UQ || field == P2DE_FIELD_RHSU || field == P2DE_FIELD_RHSL ||
                      field == P2DE_FIELD_RHSH || field == P2DE_FIELD_RESW;
  const bool flux8 = field == P2DE_FIELD_RHSXYL || field == P2DE_FIELD_RHSXYH || field == P2DE_FIELD_BF_L ||
                     field == P2DE_FIELD_BF_H;
  if (s->kpp && (state4 || flux8)) {  // the first component of each state / of each flux half
    std::vector<double> full(cnt);
    CK(cudaMemcpyAsync(full.data(), src, sizeof(double) * cnt, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    const int64_t items = state4 ? cnt / 4 : cnt / 8;
    for (int64_t i = 0; i < items; ++i) {
      if (state4) {
        out[i] = full[4 * i];
      } else {
        out[2 * i] = full[8 * i];
        out[2 * i + 1] = full[8 * i + 4];
      }
    }
    return P2DE_OK;
  }
  CK(cudaMemcpyAsync(out, src, sizeof(double) * cnt, cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  return P2DE_OK;
}

int p2de_solver_field_count(p2de_solver* s, int32_t field, int64_t* count) {
  if (!s || !count) return P2DE_ERR_INVALID_ARGUMENT;
  if (s->line) {
    const int64_t c = line_field_count(s->line, field);
    if (c < 0) return P2DE_ERR_INVALID_ARGUMENT;
    *count = c;
    return P2DE_OK;
  }
  int rc = p2de_field_count(s->N, s->K, field, count);
  if (rc != P2DE_OK) return rc;
  if (s->kpp && field != P2DE_FIELD_L_LOCAL && field != P2DE_FIELD_L && field != P2DE_FIELD_THETA_LOCAL)
    *count /= 4;
  return P2DE_OK;
}

int p2de_rhs(p2de_solver* s, double t, double dt, int32_t nstage, double* dt_out) {
  if (!s || !dt_out || nstage < 1 || nstage > 3) return P2DE_ERR_INVALID_ARGUMENT;
  CK(cudaSetDevice(s->device));
  if (s->line) {
    std::string err;
    CK(cudaMemsetAsync(s->status, 0, sizeof(int), s->stream));
    const int64_t before = s->line->launches;
    const int rc = line_rhs(s->line, t, dt, nstage, dt_out, err);
    s->launches += s->line->launches - before;
    return line_status(s, rc, err);
  }
  double sc[S_NSCAL] = {0};
  sc[S_T] = t;
  sc[S_DT_LIM] = dt;
  sc[S_DT] = dt;
  sc[S_DONE] = 0.0;
  // dtarr init of calculate_lambda_and_low_order_CFL! (low_order_graph_viscosity.jl:230)
  double dinit = std::fmin(s->prm.CFL * s->prm.dt0, s->prm.T - t);
  if (std::isnan(s->prm.CFL * s->prm.dt0) || std::isnan(s->prm.T - t)) dinit = NAN;
  unsigned long long bits;
  std::memcpy(&bits, &dinit, 8);
  CK(cudaMemcpyAsync(s->scal, sc, sizeof sc, cudaMemcpyHostToDevice, s->stream));
  CK(cudaMemcpyAsync(s->dtmin, &bits, 8, cudaMemcpyHostToDevice, s->stream));
  CK(cudaMemsetAsync(s->status, 0, sizeof(int), s->stream));
  StageArgs a = s->base;
  a.nstage = nstage;
  a.flags = flags_for(s, nstage, false, true);
  if (!(dinit > 0.0)) a.flags &= ~F_CFL;
  CK(launch_a_n1d(s->N1D, a, s->mixed, s->stream));
  CK(launch_b_n1d(s->N1D, a, s->stream));
  s->launches += a_launches(a) + 1;
  double result = dt;
  if (a.flags & F_CFL) {
    CK(cudaMemcpyAsync(&bits, s->dtmin, 8, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    std::memcpy(&result, &bits, 8);
  } else if ((a.flags & F_DO_LOW) && nstage == 1) {
    result = dinit;
  }
  // a non-positive or NaN state (kernel A's node phase), a NaN CFL candidate or a
  // non-positive CFL minimum; the reference would stop with a DomainError
  int rc = check_status(s);
  if (rc != P2DE_OK) return rc;
  if ((a.flags & F_DO_LOW) && nstage == 1 && !(result > 0.0))
    return fail(s, P2DE_ERR_BAD_DT, "stage-1 time step %g is not positive", result);
  *dt_out = result;
  return P2DE_OK;
}

static int build_graph(p2de_solver* s);

// One step from host time t: the step's CUDA graph (the launches p2de_ssp33_advance
// replays), then t, dt and the status read back.
static int step_impl(p2de_solver* s, double* t, double* dt_out) {
  int rc = build_graph(s);
  if (rc != P2DE_OK) return rc;
  CK(cudaMemcpyAsync(s->scal + S_T, t, sizeof(double), cudaMemcpyHostToDevice, s->stream));
  CK(cudaGraphLaunch(s->graph, s->stream));
  s->launches += step_launches(s);
  double sc[S_NSCAL];
  CK(cudaMemcpyAsync(sc, s->scal, sizeof sc, cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  rc = check_status(s);
  if (rc != P2DE_OK) return rc;
  if (sc[S_DONE] == 0.0) {
    *t = sc[S_T];
    *dt_out = sc[S_DT];
  } else {
    *dt_out = 0.0;
  }
  return P2DE_OK;
}

int p2de_ssp33_step(p2de_solver* s, double* t, double* dt_out) {
  if (!s || !t || !dt_out) return P2DE_ERR_INVALID_ARGUMENT;
  CK(cudaSetDevice(s->device));
  if (s->line) {
    std::string err;
    const int64_t before = s->line->launches;
    const int rc = line_step(s->line, t, dt_out, err);
    s->launches += s->line->launches - before;
    return line_status(s, rc, err);
  }
  return step_impl(s, t, dt_out);
}

// Captures one step on a private stream (the caller's stream may be the legacy
// default stream, which cannot be captured); the graph is replayed on s->stream.
static int build_graph(p2de_solver* s) {
  if (s->graph) return P2DE_OK;
  cudaStream_t cap;
  CK(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
  cudaStream_t user = s->stream;
  cudaGraph_t g = nullptr;
  s->stream = cap;
  cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
  int64_t before = s->launches;
  int rc = (e == cudaSuccess) ? enqueue_step(s) : P2DE_OK;
  cudaError_t e2 = (e == cudaSuccess) ? cudaStreamEndCapture(cap, &g) : e;
  s->launches = before;  // capture does not launch
  s->stream = user;
  cudaStreamDestroy(cap);
  if (rc != P2DE_OK) return rc;
  CK(e);
  CK(e2);
  CK(cudaGraphInstantiate(&s->graph, g, 0));
  CK(cudaGraphDestroy(g));
  return P2DE_OK;
}

int p2de_ssp33_advance(p2de_solver* s, int64_t nsteps, double* t, int64_t* steps_done) {
  if (!s || !t || nsteps < 0) return P2DE_ERR_INVALID_ARGUMENT;
  CK(cudaSetDevice(s->device));
  if (s->line) {
    std::string err;
    const int64_t before = s->line->launches;
    int64_t done = 0;
    const int rc = line_advance(s->line, nsteps, t, &done, &s->line_dt, err);
    s->launches += s->line->launches - before;
    if (steps_done) *steps_done = done;
    return line_status(s, rc, err);
  }
  int rc = build_graph(s);
  if (rc != P2DE_OK) return rc;
  double sc[S_NSCAL];
  CK(cudaMemcpyAsync(sc, s->scal, sizeof sc, cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  double steps0 = sc[S_STEPS];
  CK(cudaMemcpyAsync(s->scal + S_T, t, sizeof(double), cudaMemcpyHostToDevice, s->stream));
  for (int64_t i = 0; i < nsteps; ++i) {
    CK(cudaGraphLaunch(s->graph, s->stream));
    s->launches += step_launches(s);
  }
  CK(cudaMemcpyAsync(sc, s->scal, sizeof sc, cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  rc = check_status(s);
  *t = sc[S_T];
  if (steps_done) *steps_done = (int64_t)(sc[S_STEPS] - steps0);
  return rc;
}

int p2de_ssp33(p2de_solver* s, double* t_out, int64_t* steps_out, double* dt_last) {
  if (!s) return P2DE_ERR_INVALID_ARGUMENT;
  CK(cudaSetDevice(s->device));
  double t = s->prm.t0;
  int64_t total = 0;
  int rc = P2DE_OK;
  for (;;) {
    int64_t done = 0;
    rc = p2de_ssp33_advance(s, 64, &t, &done);
    total += done;
    if (rc != P2DE_OK || done < 64 || !(t < s->prm.T)) break;
  }
  if (t_out) *t_out = t;
  if (steps_out) *steps_out = total;
  if (s->line) {
    if (dt_last) *dt_last = s->line_dt;
    return rc;
  }
  double sc[S_NSCAL];
  CK(cudaMemcpyAsync(sc, s->scal, sizeof sc, cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  if (dt_last) *dt_last = sc[S_DT];
  return rc;
}

int p2de_profile_steps(p2de_solver* s, int64_t nsteps, double* t, double ms[3]) {
  if (!s || !t || !ms || nsteps < 1) return P2DE_ERR_INVALID_ARGUMENT;
  if (s->line) return fail(s, P2DE_ERR_UNSUPPORTED, "stage kernel timings: Dim2 solves");
  CK(cudaSetDevice(s->device));
  cudaEvent_t ev[8];
  for (int i = 0; i < 8; ++i) CK(cudaEventCreate(&ev[i]));
  double acc[3] = {0, 0, 0};
  CK(cudaMemcpyAsync(s->scal + S_T, t, sizeof(double), cudaMemcpyHostToDevice, s->stream));
  int rc = P2DE_OK;
  for (int64_t i = 0; i < nsteps && rc == P2DE_OK; ++i) {
    CK(cudaEventRecord(ev[0], s->stream));
    k_step_begin<<<1, 32, 0, s->stream>>>(s->scal, s->dtmin, s->minrec, s->status, s->prm.CFL, s->prm.dt0, s->prm.T);
    CK(cudaGetLastError());
    CK(cudaEventRecord(ev[1], s->stream));
    for (int stage = 1; stage <= 3; ++stage) {
      StageArgs a = s->base;
      a.nstage = stage;
      a.flags = flags_for(s, stage, true, false);
      CK(launch_a_n1d(s->N1D, a, s->mixed, s->stream));
      CK(cudaEventRecord(ev[2 * stage], s->stream));
      CK(launch_b_n1d(s->N1D, a, s->stream));
      CK(cudaEventRecord(ev[2 * stage + 1], s->stream));
    }
    s->launches += step_launches(s);
    CK(cudaEventSynchronize(ev[7]));
    float m;
    CK(cudaEventElapsedTime(&m, ev[0], ev[1]));
    acc[2] += m;
    for (int stage = 1; stage <= 3; ++stage) {
      CK(cudaEventElapsedTime(&m, ev[2 * stage - 1], ev[2 * stage]));
      acc[0] += m;
      CK(cudaEventElapsedTime(&m, ev[2 * stage], ev[2 * stage + 1]));
      acc[1] += m;
    }
  }
  for (int i = 0; i < 8; ++i) cudaEventDestroy(ev[i]);
  ms[0] = acc[0] / (3.0 * nsteps);
  ms[1] = acc[1] / (3.0 * nsteps);
  ms[2] = acc[2] / nsteps;
  double sc[S_NSCAL];
  CK(cudaMemcpyAsync(sc, s->scal, sizeof sc, cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  *t = sc[S_T];
  return check_status(s);
}

int p2de_set_elements_per_block(p2de_solver* s, int32_t epb) {
  if (!s) return P2DE_ERR_INVALID_ARGUMENT;
  if (s->line) return fail(s, P2DE_ERR_UNSUPPORTED, "the Line path has no elements-per-block parameter (p2de_set_layout)");
  if (epb < 1 || epb > s->geo.elems_per_block_max)
    return fail(s, P2DE_ERR_INVALID_ARGUMENT, "elements per block %d outside 1..%d", epb, s->geo.elems_per_block_max);
  CK(cudaSetDevice(s->device));
  CK(cudaStreamSynchronize(s->stream));
  s->base.epb = epb;
  if (s->graph) {
    cudaGraphExecDestroy(s->graph);
    s->graph = nullptr;
  }
  return P2DE_OK;
}

int p2de_set_layout(p2de_solver* s, int32_t layout) {
  if (!s) return P2DE_ERR_INVALID_ARGUMENT;
  if (s->line) {
    CK(cudaSetDevice(s->device));
    std::string err;
    return line_status(s, line_set_layout(s->line, layout, err), err);
  }
  if (layout != P2DE_LAYOUT_FLAT && layout != P2DE_LAYOUT_LINES_PER_WARP)
    return fail(s, P2DE_ERR_INVALID_ARGUMENT, "layout %d", layout);
  CK(cudaSetDevice(s->device));
  CK(cudaStreamSynchronize(s->stream));
  s->base.layout = layout;
  if (s->graph) {
    cudaGraphExecDestroy(s->graph);
    s->graph = nullptr;
  }
  return P2DE_OK;
}

int p2de_get_layout(p2de_solver* s, int32_t* layout) {
  if (!s || !layout) return P2DE_ERR_INVALID_ARGUMENT;
  *layout = s->line ? line_layout(s->line) : s->base.layout;
  return P2DE_OK;
}

int p2de_set_threads_per_block(p2de_solver* s, int32_t threads) {
  if (!s) return P2DE_ERR_INVALID_ARGUMENT;
  if (s->line) return fail(s, P2DE_ERR_UNSUPPORTED, "the Line path has fixed 32-thread blocks (p2de_set_layout)");
  if (threads != 64 && threads != s->geo.threads)
    return fail(s, P2DE_ERR_INVALID_ARGUMENT, "threads per block %d: 64 or %d", threads, s->geo.threads);
  CK(cudaSetDevice(s->device));
  CK(cudaStreamSynchronize(s->stream));
  s->base.threads = threads;
  if (s->graph) {
    cudaGraphExecDestroy(s->graph);
    s->graph = nullptr;
  }
  return P2DE_OK;
}

int p2de_get_threads_per_block(p2de_solver* s, int32_t* threads) {
  if (!s || !threads) return P2DE_ERR_INVALID_ARGUMENT;
  *threads = s->base.threads > 0 ? s->base.threads : s->geo.threads;
  return P2DE_OK;
}

int p2de_get_elements_per_block(p2de_solver* s, int32_t* epb, int32_t* epb_max) {
  if (!s) return P2DE_ERR_INVALID_ARGUMENT;
  if (epb) *epb = s->base.epb;
  if (epb_max) *epb_max = s->geo.elems_per_block_max;
  return P2DE_OK;
}

// Times stage kernel A (stage 2 flags, state left unchanged: no update) for each
// candidate elements-per-block and thread layout and keeps the fastest.
int p2de_autotune(p2de_solver* s, int32_t* best_epb, double* best_ms) {
  if (!s) return P2DE_ERR_INVALID_ARGUMENT;
  if (s->line) return fail(s, P2DE_ERR_UNSUPPORTED, "the Line path picks its layout by the element count (p2de_set_layout)");
  CK(cudaSetDevice(s->device));
  const int emax = s->geo.elems_per_block_max, edef = s->geo.elems_per_block;
  std::vector<int> cand;
  for (int e : {1, 2, 3, 4, 6, 8, 12, 16, 24, 32, edef})
    if (e <= emax && std::find(cand.begin(), cand.end(), e) == cand.end()) cand.push_back(e);
  // the lines-per-warp layout differs from the flat one on axis-aligned LGL elements only
  std::vector<int> layouts{P2DE_LAYOUT_FLAT};
  if (!s->gauss && !s->kpp && (flags_for(s, 2, false, false) & F_AXIS_ALIGNED))
    layouts.push_back(P2DE_LAYOUT_LINES_PER_WARP);
  int best_layout = s->base.layout;
  int best_threads = s->base.threads > 0 ? s->base.threads : s->geo.threads;
  // Gauss kernel A launches at its own fixed block size
  std::vector<int> threads{s->geo.threads};
  if (!s->gauss) threads.push_back(64);
  double sc[S_NSCAL] = {0};
  CK(cudaMemcpyAsync(sc, s->scal, sizeof sc, cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  double keep[S_NSCAL];
  std::memcpy(keep, sc, sizeof sc);
  sc[S_DONE] = 0.0;
  if (!(sc[S_DT_LIM] > 0.0)) sc[S_DT_LIM] = std::fmin(s->prm.CFL * s->prm.dt0, s->prm.T - s->prm.t0);
  CK(cudaMemcpyAsync(s->scal, sc, sizeof sc, cudaMemcpyHostToDevice, s->stream));
  int best = edef;
  double bms = 1e30;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  // the timings; whatever they return, the events go and the scalars come back below
  auto timings = [&]() -> int {
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  for (int th : threads)
  for (int lay : layouts)
  for (int e : cand) {
    StageArgs a = s->base;
    a.epb = e;
    a.layout = lay;
    a.threads = th;
    a.nstage = 2;
    a.flags = flags_for(s, 2, false, false);
    float tot = 0.f;
    for (int rep = 0; rep < 4; ++rep) {
      CK(cudaEventRecord(e0, s->stream));
      CK(launch_a_n1d(s->N1D, a, s->mixed, s->stream));
      CK(cudaEventRecord(e1, s->stream));
      CK(cudaEventSynchronize(e1));
      float ms;
      CK(cudaEventElapsedTime(&ms, e0, e1));
      if (rep > 0) tot += ms;  // first launch warms up
    }
    s->launches += 4 * a_launches(a);
    double ms = tot / 3.0;
    if (ms < bms) {
      bms = ms;
      best = e;
      best_layout = lay;
      best_threads = th;
    }
  }
  return P2DE_OK;
  };
  const int rt = timings();
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  CK(cudaMemcpyAsync(s->scal, keep, sizeof keep, cudaMemcpyHostToDevice, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  if (rt != P2DE_OK) return rt;
  int rc = p2de_set_layout(s, best_layout);
  if (rc == P2DE_OK) rc = p2de_set_threads_per_block(s, best_threads);
  if (rc == P2DE_OK) rc = p2de_set_elements_per_block(s, best);
  if (best_epb) *best_epb = best;
  if (best_ms) *best_ms = bms;
  return rc;
}

int p2de_read_counters(p2de_solver* s, uint64_t out[1], int32_t reset) {
  if (!s || !out) return P2DE_ERR_INVALID_ARGUMENT;
  CK(cudaSetDevice(s->device));
  unsigned long long c[1];
  CK(cudaMemcpyAsync(c, s->counters, sizeof c, cudaMemcpyDeviceToHost, s->stream));
  if (reset) CK(cudaMemsetAsync(s->counters, 0, sizeof(unsigned long long) * 8, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  out[0] = c[0];
  return P2DE_OK;
}

int p2de_device_ptr(p2de_solver* s, int32_t field, void** dptr) {
  if (!s || !dptr) return P2DE_ERR_INVALID_ARGUMENT;
  switch (field) {
    case P2DE_FIELD_UQ: *dptr = s->Uq; break;
    case P2DE_FIELD_RHSU: *dptr = s->rhsU; break;
    case P2DE_FIELD_RHSL: *dptr = s->rhsL; break;
    case P2DE_FIELD_RHSH: *dptr = s->rhsH; break;
    case P2DE_FIELD_RESW: *dptr = s->resW; break;
    case P2DE_FIELD_L_LOCAL: *dptr = s->line ? s->line->Lloc : s->Lfin; break;
    default: return fail(s, P2DE_ERR_INVALID_ARGUMENT, "no device pointer for field %d", field);
  }
  return P2DE_OK;
}

int p2de_set_stream(p2de_solver* s, void* stream) {
  if (!s) return P2DE_ERR_INVALID_ARGUMENT;
  CK(cudaSetDevice(s->device));
  CK(cudaStreamSynchronize(s->stream));
  if (s->graph) {
    cudaGraphExecDestroy(s->graph);
    s->graph = nullptr;
  }
  if (s->own_stream) cudaStreamDestroy(s->stream);
  s->own_stream = false;
  s->stream = (cudaStream_t)stream;
  if (s->line) s->line->stream = s->stream;
  return P2DE_OK;
}

int p2de_launch_count(p2de_solver* s, int64_t* count) {
  if (!s || !count) return P2DE_ERR_INVALID_ARGUMENT;
  *count = s->launches;
  return P2DE_OK;
}

int p2de_min_rho_rhoe(p2de_solver* s, double* min_rho, double* min_rhoe) {
  if (!s || !min_rho || !min_rhoe) return P2DE_ERR_INVALID_ARGUMENT;
  CK(cudaSetDevice(s->device));
  long long init[2] = {0x7ff0000000000000LL, 0x7ff0000000000000LL};
  CK(cudaMemcpyAsync(s->minbuf, init, sizeof init, cudaMemcpyHostToDevice, s->stream));
  size_t nodes = (size_t)s->Nq * s->K;
  int grid = (int)std::min<size_t>((nodes + 255) / 256, 152 * 8);
  k_min_rho_rhoe<<<grid, 256, 0, s->stream>>>(s->Uq, nodes, s->minbuf);
  CK(cudaGetLastError());
  s->launches += 1;
  long long outk[2];
  CK(cudaMemcpyAsync(outk, s->minbuf, sizeof outk, cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  *min_rho = key_to_double(outk[0]);
  *min_rhoe = key_to_double(outk[1]);
  return P2DE_OK;
}

namespace {

int diag_prepare(p2de_solver* s, bool exact) {
  if (!s->diag_partial) {
    cudaDeviceProp prop;
    CK(cudaGetDeviceProperties(&prop, s->device));
    s->diag_nblocks = diag_blocks(prop.multiProcessorCount);
    CK(dalloc(s, &s->diag_partial, (size_t)24 * s->diag_nblocks));
    CK(dalloc(s, &s->diag_out, 24));
  }
  if (exact && !s->exact) CK(dalloc(s, &s->exact, (size_t)4 * s->Nq * s->K));
  return P2DE_OK;
}

const double* device_wq(const p2de_solver* s) {
  if (s->line)
    return reinterpret_cast<const double*>(reinterpret_cast<const char*>(s->line->ops) + offsetof(LineOps, wq));
  const OpTable* t = table_of(s);
  return reinterpret_cast<const double*>(reinterpret_cast<const char*>(t) + offsetof(OpTable, wq));
}

}  // namespace

// check_conservation (src/dg/utils.jl:1-12) on the device
int p2de_check_conservation(p2de_solver* s, double totals[4], double* sum) {
  if (!s) return P2DE_ERR_INVALID_ARGUMENT;
  CK(cudaSetDevice(s->device));
  int rc = diag_prepare(s, false);
  if (rc != P2DE_OK) return rc;
  CK(launch_weighted_sum(s->Uq, s->geom, device_wq(s), s->Nq, (long long)s->Nq * s->K, s->diag_nblocks,
                         s->diag_partial, s->diag_out, s->stream));
  s->launches += 2;
  double t[4];
  CK(cudaMemcpyAsync(t, s->diag_out, sizeof t, cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  if (s->line) {  // (rho, rhou, E): the Line state's y-momentum slot is 0
    t[2] = t[3];
    t[3] = 0.0;
    if (sum) *sum = (t[0] + t[1]) + t[2];
  } else if (sum) {
    *sum = ((t[0] + t[1]) + t[2]) + t[3];
  }
  if (totals)
    for (int c = 0; c < 4; ++c) totals[c] = t[c];
  return P2DE_OK;
}

// calculate_error (src/dg/postprocess.jl:1-46) on the device, against exact conservative
// values at the nodes (host array in the layout of Uq)
int p2de_calculate_error(p2de_solver* s, const double* exact_Uq, double out[3]) {
  if (!s || !exact_Uq || !out) return P2DE_ERR_INVALID_ARGUMENT;
  CK(cudaSetDevice(s->device));
  int rc = diag_prepare(s, true);
  if (rc != P2DE_OK) return rc;
  const size_t n = (size_t)4 * s->Nq * s->K;
  std::vector<double> full;
  if (s->kpp) {  // one component per node
    full.assign(n, 0.0);
    for (size_t i = 0; i < n / 4; ++i) full[4 * i] = exact_Uq[i];
    exact_Uq = full.data();
  } else if (s->line) {  // (rho, rhou, E) per node
    full.assign(n, 0.0);
    for (size_t i = 0; i < n / 4; ++i) {
      full[4 * i] = exact_Uq[3 * i];
      full[4 * i + 1] = exact_Uq[3 * i + 1];
      full[4 * i + 3] = exact_Uq[3 * i + 2];
    }
    exact_Uq = full.data();
  }
  CK(cudaMemcpyAsync(s->exact, exact_Uq, sizeof(double) * n, cudaMemcpyHostToDevice, s->stream));
  CK(launch_error_norms(s->Uq, s->exact, s->geom, device_wq(s), s->Nq, (long long)s->Nq * s->K, s->diag_nblocks,
                        s->diag_partial, s->diag_out, s->stream));
  s->launches += 2;
  double v[24];
  CK(cudaMemcpyAsync(v, s->diag_out, sizeof v, cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  double L1 = 0.0, L2 = 0.0, Linf = 0.0;
  for (int c = 0; c < 4; ++c)
    if (v[20 + c] > 1e-14) {
      L1 += v[0 + c] / v[12 + c];
      L2 += std::sqrt(v[4 + c]) / std::sqrt(v[16 + c]);
      Linf += v[8 + c] / v[20 + c];
    }
  out[0] = L1;
  out[1] = L2;
  out[2] = Linf;
  return P2DE_OK;
}

int p2de_stage_minima(p2de_solver* s, double out[6]) {
  if (!s || !out) return P2DE_ERR_INVALID_ARGUMENT;
  CK(cudaSetDevice(s->device));
  long long k[6];
  const long long* rec = s->line ? s->line->minrec : s->minrec;
  CK(cudaMemcpyAsync(k, rec, sizeof k, cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  for (int i = 0; i < 6; ++i) out[i] = key_to_double(k[i]);
  return P2DE_OK;
}

int p2de_last_error(p2de_solver* s, char* buf, size_t len) {
  if (!buf || len == 0) return P2DE_ERR_INVALID_ARGUMENT;
  std::string m;
  if (s)
    m = s->err;
  else {
    std::lock_guard<std::mutex> lk(g_err_mu);
    m = g_last_create_error;
  }
  std::snprintf(buf, len, "%s", m.c_str());
  return P2DE_OK;
}

}  // extern "C"
