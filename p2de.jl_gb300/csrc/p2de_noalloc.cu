// p2de_rhs_noalloc: the right-hand side evaluation (stage kernels A and B without the
// stage update) with every piece of scratch memory in one file-scope device array,
// for callers that cannot allocate device memory. Some hosts cannot call cudaMalloc
// at the moment they need a right-hand side: a Julia or serving process whose device
// memory is reserved up front by its own pool allocator (a further cudaMalloc would
// fail or break the budget the pool enforces), or an application that allows device
// allocation only during its start-up. This entry point only launches kernels and copies
// a few bytes of parameters and results; it calls no cudaMalloc, cudaFree or allocating
// library routine. It synchronizes its stream before returning (the index check, the
// status word and dt are read back to the host).
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>

#include "../../include/p2de.h"
#include "p2de_args.h"
#include "p2de_launch.h"
#include "p2de_tables.h"

using namespace p2de;

namespace {

constexpr size_t kScratchDoubles = (size_t)P2DE_NOALLOC_SCRATCH_BYTES / sizeof(double);

// Scratch shared by every call on a device, kept until the process exits. Calls that
// overlap on the GPU (two streams, or a call issued before the previous one finished)
// race on it.
static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

// header slots of the scratch, in doubles
constexpr size_t H_SCAL = 0;         // S_NSCAL doubles
constexpr size_t H_DTMIN = 8;        // 1 unsigned long long
constexpr size_t H_STATUS = 9;       // 1 int (its own 8-byte slot)
constexpr size_t H_BADIDX = 10;      // 1 int: index checks of the last call
constexpr size_t H_MINREC = 16;      // 6 long long
constexpr size_t H_COUNTERS = 24;    // 8 unsigned long long
constexpr size_t H_TABLE = 64;       // OpTable
constexpr size_t kTableDoubles = (sizeof(OpTable) + 255) / 256 * 256 / sizeof(double);
constexpr size_t H_DATA = H_TABLE + kTableDoubles;

struct DeviceState {
  bool ready = false;
  double* scratch = nullptr;  // device address of g_noalloc_scratch on this device
  // the OpTable the scratch holds: build_op_table depends on the degree and on ZEROTOL
  // (entries below it are set to zero), so both are its key
  int table_N = 0;
  uint64_t table_zerotol_bits = 0;
};
std::mutex g_mu;
DeviceState g_dev[64];

// Checks the caller's index arrays: exterior indices in range, boundary codes known,
// boundary indices within Ival / xyS. Sets *bad to 1 on any violation.
__global__ void k_check_indices(const int32_t* nbr, const int8_t* bc, const int32_t* bcidx, long long nfk,
                                long long nI, long long nS, int* bad) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nfk; i += (long long)gridDim.x * blockDim.x) {
    int lin = nbr[i];
    int code = bc[i];
    bool ok = lin >= 0 && lin < nfk && code >= BC_INTERIOR && code <= BC_SHOCK;
    if (ok && code == BC_INFLOW) ok = bcidx != nullptr && bcidx[i] >= 0 && bcidx[i] < nI;
    if (ok && code == BC_SHOCK) ok = bcidx != nullptr && bcidx[i] >= 0 && bcidx[i] < nS;
    if (!ok) atomicOr(bad, 1);
  }
}

size_t data_doubles_per_elem(int n1d) {
  size_t nq = (size_t)n1d * n1d, nsf = (size_t)n1d * (n1d + 1);
  // Lpre, Lfin (3 stages), subcell fluxes, rhsL, rhsH
  return 2 * nsf + 3 * 2 * nsf + 16 * nsf + 4 * nq + 4 * nq;
}

cudaError_t prepare(int n1d, StageGeometry* geo) {
  switch (n1d) {
    case 2: return stage_prepare<2>(geo);
    case 3: return stage_prepare<3>(geo);
    case 4: return stage_prepare<4>(geo);
    case 5: return stage_prepare<5>(geo);
    case 6: return stage_prepare<6>(geo);
  }
  return cudaErrorInvalidValue;
}
cudaError_t launch_a(int n1d, const StageArgs& a, bool mixed, cudaStream_t st) {
  switch (n1d) {
    case 2: return launch_stage_a<2>(a, mixed, st);
    case 3: return launch_stage_a<3>(a, mixed, st);
    case 4: return launch_stage_a<4>(a, mixed, st);
    case 5: return launch_stage_a<5>(a, mixed, st);
    case 6: return launch_stage_a<6>(a, mixed, st);
  }
  return cudaErrorInvalidValue;
}
cudaError_t launch_b(int n1d, const StageArgs& a, cudaStream_t st) {
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

extern "C" int p2de_noalloc_max_elements(int32_t N, int64_t* K_max) {
  if (N < 1 || N > 5 || !K_max) return P2DE_ERR_INVALID_ARGUMENT;
  *K_max = (int64_t)((kScratchDoubles - H_DATA) / data_doubles_per_elem(N + 1));
  return P2DE_OK;
}

extern "C" int p2de_rhs_noalloc(const p2de_param* prm, const p2de_device_mesh* mesh, const double* Uq, double t,
                                double dt, int32_t nstage, double* rhsU, double* dt_out, void* stream) {
  if (!prm || !mesh || !Uq || !rhsU || !dt_out || !mesh->geom || !mesh->nbr || !mesh->bc) return P2DE_ERR_INVALID_ARGUMENT;
  if (prm->N < 1 || prm->N > 5 || prm->K < 1 || nstage < 1 || nstage > 3) return P2DE_ERR_INVALID_ARGUMENT;
  if (prm->low_order_surface_flux != P2DE_FLUX_LAX_FRIEDRICHS_ON_NODAL_VAL ||
      prm->high_order_surface_flux != P2DE_FLUX_LAX_FRIEDRICHS_ON_PROJECTED_VAL || prm->rhs_type < 0 ||
      prm->rhs_type > 2 || prm->bound_type < 0 || prm->bound_type > 1 || prm->shock_capture < 0 ||
      prm->shock_capture > 1 || prm->rhs_limiter != P2DE_LIMITER_SUBCELL ||
      prm->approximation_basis != P2DE_BASIS_LOBATTO || prm->equation != P2DE_EQUATION_COMPRESSIBLE_EULER)
    return P2DE_ERR_UNSUPPORTED;
  const int n1d = prm->N + 1;
  const size_t K = (size_t)prm->K;
  if (H_DATA + K * data_doubles_per_elem(n1d) > kScratchDoubles) return P2DE_ERR_BUDGET;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return P2DE_ERR_NO_DEVICE;
  cudaStream_t st = (cudaStream_t)stream;
  double* scr = nullptr;
  StageGeometry geo{};
  {
    // set-up, once per device, with that device current: the address of the scratch
    // array (a host-side symbol is not a device address) and the kernels' shared-memory
    // limits; the first call on a device should therefore come before any stream capture
    // on that device
    std::lock_guard<std::mutex> lk(g_mu);
    DeviceState& d = g_dev[dev];
    if (!d.ready) {
      void* ptr = nullptr;
      if (cudaGetSymbolAddress(&ptr, g_noalloc_scratch) != cudaSuccess || !ptr) return P2DE_ERR_CUDA;
      d.scratch = (double*)ptr;
      d.ready = true;
    }
    if (prepare(n1d, &geo) != cudaSuccess) return P2DE_ERR_CUDA;
    scr = d.scratch;
    uint64_t zbits;
    std::memcpy(&zbits, &prm->ZEROTOL, sizeof zbits);
    if (d.table_N != prm->N || d.table_zerotol_bits != zbits) {
      OpTable tab;
      if (build_op_table(prm->N, prm->ZEROTOL, &tab) != 0) return P2DE_ERR_INVALID_ARGUMENT;
      d.table_N = 0;  // invalid until the copy below has completed
      if (cudaMemcpyAsync(scr + H_TABLE, &tab, sizeof tab, cudaMemcpyHostToDevice, st) != cudaSuccess ||
          cudaStreamSynchronize(st) != cudaSuccess)
        return P2DE_ERR_CUDA;
      d.table_N = prm->N;
      d.table_zerotol_bits = zbits;
    }
  }
  const size_t nsf = geo.nsf, nq = (size_t)n1d * n1d;
  const long long nfk = (long long)K * 4 * n1d;
  // everything that must start from a known value is written on every call
  double hdr[16] = {0};
  hdr[S_T] = t;
  hdr[S_DT_LIM] = dt;
  hdr[S_DT] = dt;
  hdr[S_DONE] = 0.0;
  double dinit = std::fmin(prm->CFL * prm->dt0, prm->T - t);
  std::memcpy(&hdr[H_DTMIN], &dinit, 8);  // initial value of the CFL minimum
  // H_STATUS and H_BADIDX stay zero
  if (cudaMemcpyAsync(scr, hdr, sizeof hdr, cudaMemcpyHostToDevice, st) != cudaSuccess) return P2DE_ERR_CUDA;
  if (cudaMemsetAsync(scr + H_COUNTERS, 0, 8 * sizeof(double), st) != cudaSuccess) return P2DE_ERR_CUDA;
  int* status = (int*)(scr + H_STATUS);
  int* badidx = (int*)(scr + H_BADIDX);
  k_check_indices<<<(int)std::min<long long>((nfk + 255) / 256, 1024), 256, 0, st>>>(mesh->nbr, mesh->bc, mesh->bcidx,
                                                                                     nfk, mesh->nI, mesh->nS, badidx);
  if (cudaGetLastError() != cudaSuccess) return P2DE_ERR_CUDA;
  int bad = 0;
  if (cudaMemcpyAsync(&bad, badidx, sizeof bad, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return P2DE_ERR_CUDA;
  if (bad) return P2DE_ERR_INVALID_ARGUMENT;

  StageArgs a{};
  a.K = prm->K;
  a.epb = geo.elems_per_block;
  a.nstage = nstage;
  int f = 0;
  switch (prm->rhs_type) {
    case P2DE_RHS_LOW_ORDER_POSITIVITY: f |= F_DO_LOW | F_RHSU_FROM_L; break;
    case P2DE_RHS_ENTROPY_STABLE: f |= F_DO_HIGH | F_RHSU_FROM_H; break;
    default: f |= F_DO_LOW | F_DO_HIGH | F_DO_LIMIT; break;
  }
  if ((f & F_DO_LOW) && nstage == 1 && dinit > 0.0) f |= F_CFL;
  if (prm->reference_semantics) f |= F_REF_SEM;
  if (prm->bound_type == P2DE_BOUND_POSITIVITY_AND_CELL_ENTROPY) f |= F_CELL_ENTROPY;
  if (mesh->axis_aligned) f |= F_AXIS_ALIGNED;
  if (prm->precision == P2DE_PRECISION_MIXED_ACC64) f |= F_ACC64;
  if (prm->shock_capture == 1 && (f & F_DO_LIMIT)) f |= F_SHOCK;
  a.flags = f;
  set_shock_capture(a, prm->N, prm->shock_capture_a, prm->shock_capture_c);
  a.ops = (const OpTable*)(scr + H_TABLE);
  a.Uq = const_cast<double*>(Uq);
  a.resW = nullptr;
  a.geom = mesh->geom;
  a.nbr = mesh->nbr;
  a.bc = mesh->bc;
  a.bcidx = mesh->bcidx;
  a.Ival = mesh->Ival;
  a.xyS = mesh->xyS;
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
  double* data = scr + H_DATA;
  a.Lpre = data;
  a.Lfin = a.Lpre + 2 * nsf * K;
  a.fbar = a.Lfin + 3 * 2 * nsf * K;
  a.rhsL = a.fbar + 16 * nsf * K;
  a.rhsH = a.rhsL + 4 * nq * K;
  a.rhsU = rhsU;
  a.rhsxyL = a.rhsxyH = a.BFL = a.BFH = nullptr;
  a.scal = scr + H_SCAL;
  a.dtmin_bits = (unsigned long long*)(scr + H_DTMIN);
  a.minrec = (long long*)(scr + H_MINREC);
  a.status = status;
  a.counters = (unsigned long long*)(scr + H_COUNTERS);
  if (launch_a(n1d, a, prm->precision != P2DE_PRECISION_FP64, st) != cudaSuccess) return P2DE_ERR_CUDA;
  if (launch_b(n1d, a, st) != cudaSuccess) return P2DE_ERR_CUDA;
  double dtres = dt;
  int stv = 0;
  if (cudaMemcpyAsync(&stv, status, sizeof stv, cudaMemcpyDeviceToHost, st) != cudaSuccess) return P2DE_ERR_CUDA;
  if (f & F_CFL) {
    if (cudaMemcpyAsync(&dtres, scr + H_DTMIN, sizeof dtres, cudaMemcpyDeviceToHost, st) != cudaSuccess)
      return P2DE_ERR_CUDA;
  } else if ((f & F_DO_LOW) && nstage == 1) {
    dtres = dinit;
  }
  if (cudaStreamSynchronize(st) != cudaSuccess) return P2DE_ERR_CUDA;
  if (stv & (ST_NOT_POSITIVE | ST_NAN)) return P2DE_ERR_NOT_POSITIVE;
  if (stv & ST_BAD_DT) return P2DE_ERR_BAD_DT;
  *dt_out = dtres;
  return P2DE_OK;
}
