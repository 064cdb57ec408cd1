// Batches of independent solves (uneven mesh sizes and degrees) advanced together by
// one persistent launch per RK stage, and a continuous-batching server on top.
//
// Device memory comes from one pool allocated at creation (the HBM budget); a solve is
// admitted when its arrays fit in the pool, and its memory returns to the pool when it
// is removed. Per-solve time, dt, status and stage minima live in slot-indexed arrays,
// so every solve keeps its own CFL step and final time while the stages run in
// lockstep. The 7 launches of a step are captured once in a CUDA graph that reads the
// work list and the solve descriptors from device memory, so changing the batch's
// membership does not need a new capture.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/p2de.h"
#include "p2de_args.h"
#include "p2de_batch_kernels.cuh"
#include "p2de_batch_launch.h"
#include "p2de_launch.h"
#include "p2de_tables.h"

using namespace p2de;

namespace {

constexpr size_t kAlign = 256;
size_t align_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

// Best-fit allocator over one device allocation, with coalescing of freed blocks.
class Pool {
 public:
  char* base = nullptr;
  size_t cap = 0, in_use = 0;
  std::map<size_t, size_t> free_;  // offset -> size
  std::map<size_t, size_t> used_;

  cudaError_t init(size_t bytes) {
    cap = align_up(bytes);
    cudaError_t e = cudaMalloc(&base, cap);
    if (e != cudaSuccess) return e;
    free_[0] = cap;
    return cudaSuccess;
  }
  void release() {
    if (base) cudaFree(base);
    base = nullptr;
  }
  bool alloc(size_t bytes, size_t* off) {
    bytes = align_up(bytes);
    auto best = free_.end();
    for (auto it = free_.begin(); it != free_.end(); ++it)
      if (it->second >= bytes && (best == free_.end() || it->second < best->second)) best = it;
    if (best == free_.end()) return false;
    *off = best->first;
    size_t rest = best->second - bytes;
    free_.erase(best);
    if (rest) free_[*off + bytes] = rest;
    used_[*off] = bytes;
    in_use += bytes;
    return true;
  }
  void release_block(size_t off) {
    auto it = used_.find(off);
    if (it == used_.end()) return;
    size_t sz = it->second;
    used_.erase(it);
    in_use -= sz;
    auto nx = free_.lower_bound(off);
    if (nx != free_.end() && off + sz == nx->first) {
      sz += nx->second;
      free_.erase(nx);
    }
    auto pv = free_.lower_bound(off);
    if (pv != free_.begin()) {
      --pv;
      if (pv->first + pv->second == off) {
        pv->second += sz;
        return;
      }
    }
    free_[off] = sz;
  }
  size_t largest_free() const {
    size_t m = 0;
    for (auto& kv : free_) m = std::max(m, kv.second);
    return m;
  }
};

// offsets of a solve's arrays inside its pool block
struct Layout {
  size_t Uq, resW, rhsU, rhsL, rhsH, geom, geomx, fbar, Lpre, Lfin, Ival, xyS, nbr, bcidx, bc, rhoL, Lelem, phimin,
      total;
};

Layout layout_for(const p2de_param& p, int64_t nI, int64_t nS) {
  const size_t n = p.N + 1, Nq = n * n, Nfp = 4 * n, NSF = n * (n + 1), K = (size_t)p.K;
  const bool other = p.rhs_type != P2DE_RHS_ES_LIMITED_LOW_ORDER_POS;
  Layout L{};
  size_t o = 0;
  auto take = [&](size_t bytes) {
    size_t at = o;
    o += align_up(bytes > 0 ? bytes : 8);
    return at;
  };
  L.Uq = take(8 * 4 * Nq * K);
  L.resW = take(8 * 4 * Nq * K);
  L.rhsU = take(8 * 4 * Nq * K);
  L.rhsL = take(other ? 8 * 4 * Nq * K : 8);
  L.rhsH = take(other ? 8 * 4 * Nq * K : 8);
  L.geom = take(8 * 5 * K);
  L.geomx = take(8 * 16 * K);
  L.fbar = take(8 * 16 * NSF * K);
  L.Lpre = take(8 * 2 * NSF * K);
  L.Lfin = take(8 * 3 * 2 * NSF * K);
  L.Ival = take(8 * 4 * (size_t)std::max<int64_t>(nI, 1));
  L.xyS = take(8 * 2 * (size_t)std::max<int64_t>(nS, 1));
  L.nbr = take(4 * Nfp * K);
  L.bcidx = take(4 * Nfp * K);
  L.bc = take(Nfp * K);
  // TVD bounds: the low-order densities; Zhang-Shu: the per-element factors of the three
  // stages; min-entropy bounds: the initial minimum of phi
  const bool tvd = p.rhs_limiter == P2DE_LIMITER_SUBCELL && (bound_flags(p.bound_type) & F_TVD);
  L.rhoL = take(tvd ? 8 * Nq * K : 8);
  L.Lelem = take(p.rhs_limiter == P2DE_LIMITER_ZHANG_SHU ? 8 * 3 * K : 8);
  L.phimin = take(8);
  L.total = o;
  return L;
}

// The flags of a member as the one-solve path sets them for its stage kernels (without
// the stage-dependent F_CFL, F_UPDATE and the debug outputs), so that each member runs the
// same arithmetic in the batch as alone.
int member_flags(const p2de_param& p, bool axis_aligned, int precision) {
  int f = 0;
  switch (p.rhs_type) {
    case P2DE_RHS_LOW_ORDER_POSITIVITY: f |= F_DO_LOW | F_RHSU_FROM_L; break;
    case P2DE_RHS_ENTROPY_STABLE: f |= F_DO_HIGH | F_RHSU_FROM_H; break;
    default: f |= F_DO_LOW | F_DO_HIGH | F_DO_LIMIT; break;
  }
  if (axis_aligned) f |= F_AXIS_ALIGNED;
  if (f & F_DO_LIMIT) {
    if (p.rhs_limiter == P2DE_LIMITER_ZHANG_SHU) {
      f = (f & ~F_DO_LIMIT) | F_ZHANG_SHU;
    } else {
      f |= bound_flags(p.bound_type);
      if (p.reference_semantics && !(f & F_MIN_ENTROPY)) f |= F_REF_SEM;
    }
  }
  if (precision == P2DE_PRECISION_MIXED_ACC64) f |= F_ACC64;
  if (p.shock_capture == 1 && (f & (F_DO_LIMIT | F_ZHANG_SHU))) f |= F_SHOCK;
  if (p.low_order_surface_flux == P2DE_FLUX_LAX_FRIEDRICHS_ON_PROJECTED_VAL) f |= F_LFPROJ;
  return f;
}

struct Slot {
  bool active = false;
  p2de_param prm{};
  int n1d = 0;
  int flags = 0;  // member_flags
  size_t off = 0;
  Layout lay{};
};

// Task segments of a batch: the members' tasks for the plain and the EXT instantiation of
// kernel A, then the same members' tasks again for the low-only pass of the TVD bounds.
// Kernel B runs over segments 0 and 1, which are contiguous.
enum : int { SEG_PLAIN = 0, SEG_EXT = 1, SEG_LOW_PLAIN = 2, SEG_LOW_EXT = 3, NSEG = 4 };

double now_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

}  // namespace

struct p2de_batch {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool mixed = false;
  int precision = 0;
  Pool pool;
  int max_solves = 0;
  std::vector<Slot> slots;
  std::vector<uint8_t> active;
  StageArgs* d_solves = nullptr;
  uint8_t* d_active = nullptr;
  BatchTask* d_tasks = nullptr;
  int* d_ntasks = nullptr;
  unsigned* d_counters = nullptr;
  double* d_scal = nullptr;
  unsigned long long* d_dtmin = nullptr;
  long long* d_minrec = nullptr;
  int* d_status = nullptr;
  unsigned long long* d_work = nullptr;
  // operator tables by ZEROTOL (build_op_table drops entries at or below it): group g
  // holds N1D = 2..6 for the value whose bits are table_zerotol[g]
  OpTable* d_tables = nullptr;
  std::vector<uint64_t> table_zerotol;
  int task_cap = 0;
  int sms = 0;
  int grid_a = 0, grid_x = 0, grid_b = 0;
  // launch shared memory of the captured graph: plain and EXT kernel A, kernel B
  size_t smem_a = 0, smem_x = 0, smem_b = 0;
  int seg_off[NSEG] = {}, seg_cnt[NSEG] = {};  // task segments (offsets into d_tasks)
  bool phi_min = false;                         // some member needs the initial min of phi
  int epb[kMaxN1D + 1] = {};     // elements per block per N1D
  int layout[kMaxN1D + 1] = {};  // thread layout (p2de_layout) per N1D
  cudaGraphExec_t graph = nullptr;
  bool tasks_dirty = true;
  int64_t launches = 0;
  std::string err;
  std::vector<void*> allocs;
};

namespace {

constexpr int kBatchTableGroups = 8;  // distinct ZEROTOL values one batch can hold

// The table group of b for ZEROTOL value z, built and uploaded on first use; -1 when all
// groups are taken or the upload fails.
int batch_table_group(p2de_batch* b, double z) {
  uint64_t bits;
  std::memcpy(&bits, &z, sizeof bits);
  for (size_t g = 0; g < b->table_zerotol.size(); ++g)
    if (b->table_zerotol[g] == bits) return (int)g;
  if ((int)b->table_zerotol.size() >= kBatchTableGroups) return -1;
  std::vector<OpTable> tabs(kMaxN1D - 1);
  for (int N = 1; N < kMaxN1D; ++N) build_op_table(N, z, &tabs[N - 1]);
  const size_t g = b->table_zerotol.size();
  if (cudaMemcpyAsync(b->d_tables + g * (kMaxN1D - 1), tabs.data(), sizeof(OpTable) * tabs.size(),
                      cudaMemcpyHostToDevice, b->stream) != cudaSuccess ||
      cudaStreamSynchronize(b->stream) != cudaSuccess)
    return -1;
  b->table_zerotol.push_back(bits);
  return (int)g;
}

int bfail(p2de_batch* b, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (b) b->err = buf;
  return code;
}

#define BCK(call)                                                                                   \
  do {                                                                                              \
    cudaError_t e_ = (call);                                                                        \
    if (e_ != cudaSuccess) return bfail(b, P2DE_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

template <typename T>
cudaError_t balloc(p2de_batch* b, T** p, size_t count) {
  void* q = nullptr;
  cudaError_t e = cudaMalloc(&q, sizeof(T) * std::max<size_t>(count, 1));
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(q, 0, sizeof(T) * std::max<size_t>(count, 1), b->stream);
  if (e != cudaSuccess) return e;
  b->allocs.push_back(q);
  *p = (T*)q;
  return cudaSuccess;
}

int validate_solve(const p2de_param* p, const p2de_mesh* m, std::string& why) {
  char buf[256];
  if (!p || !m || !m->geom || !m->mapP) {
    why = "null param/mesh/geom/mapP";
    return P2DE_ERR_INVALID_ARGUMENT;
  }
  if (p->N < 1 || p->N > 5 || p->K < 1) {
    why = "N outside 1..5 or K < 1";
    return P2DE_ERR_INVALID_ARGUMENT;
  }
  // every bound and RHS limiter of the one-solve path on LGL nodes for 2D Euler; Gauss
  // collocation (its face projection and interface launches) and KPP run one solve per handle
  if ((p->low_order_surface_flux != P2DE_FLUX_LAX_FRIEDRICHS_ON_NODAL_VAL &&
       p->low_order_surface_flux != P2DE_FLUX_LAX_FRIEDRICHS_ON_PROJECTED_VAL) ||
      p->high_order_surface_flux != P2DE_FLUX_LAX_FRIEDRICHS_ON_PROJECTED_VAL || p->rhs_type < 0 || p->rhs_type > 2 ||
      p->bound_type < 0 || p->bound_type > 9 || p->shock_capture < 0 || p->shock_capture > 1 ||
      (p->rhs_limiter != P2DE_LIMITER_SUBCELL && p->rhs_limiter != P2DE_LIMITER_ZHANG_SHU)) {
    why = "unsupported method";
    return P2DE_ERR_UNSUPPORTED;
  }
  if (p->approximation_basis != P2DE_BASIS_LOBATTO || p->equation != P2DE_EQUATION_COMPRESSIBLE_EULER) {
    why = "batches run 2D Euler on LGL nodes; GaussCollocation and KPP solves run one per handle";
    return P2DE_ERR_UNSUPPORTED;
  }
  const int64_t nfk = (int64_t)4 * (p->N + 1) * p->K;
  for (int64_t i = 0; i < nfk; ++i)
    if (m->mapP[i] < 1 || m->mapP[i] > nfk) {
      std::snprintf(buf, sizeof buf, "mapP[%lld] out of range", (long long)i);
      why = buf;
      return P2DE_ERR_INVALID_ARGUMENT;
    }
  auto chk = [&](const int64_t* a, int64_t n) {
    if (n < 0 || (n > 0 && !a)) return false;
    for (int64_t i = 0; i < n; ++i)
      if (a[i] < 1 || a[i] > nfk) return false;
    return true;
  };
  if (!chk(m->mapI, m->nI) || !chk(m->mapO, m->nO) || !chk(m->mapW, m->nW) || !chk(m->mapS, m->nS) ||
      (m->nI > 0 && !m->Ival) || (m->nS > 0 && !m->xyS)) {
    why = "boundary lists";
    return P2DE_ERR_INVALID_ARGUMENT;
  }
  for (int64_t k = 0; k < p->K; ++k)
    if (!(m->geom[5 * k] > 0.0)) {
      why = "J not positive";
      return P2DE_ERR_INVALID_ARGUMENT;
    }
  return P2DE_OK;
}

// The tasks of one member: elements in runs of the degree's elements per block.
void member_tasks(const p2de_batch* b, int s, std::vector<BatchTask>& t) {
  const Slot& sl = b->slots[s];
  const int E = b->epb[sl.n1d];
  for (int k0 = 0; k0 < sl.prm.K; k0 += E) t.push_back(BatchTask{s, k0, sl.n1d, E, b->layout[sl.n1d]});
}

// The task list in its segments, largest tasks first within each (work per task grows
// with elements * N1D^3), and the kernels' shared memory for each instantiation.
std::vector<BatchTask> build_tasks(p2de_batch* b, size_t* smem_a, size_t* smem_x, size_t* smem_b) {
  std::vector<BatchTask> seg[NSEG];
  *smem_a = *smem_x = *smem_b = 0;
  for (int s = 0; s < b->max_solves; ++s) {
    const Slot& sl = b->slots[s];
    if (!sl.active) continue;
    const bool ext = sl.flags & kExtFlags, tvd = sl.flags & F_TVD;
    const int E = b->epb[sl.n1d];
    (ext ? *smem_x : *smem_a) = std::max(ext ? *smem_x : *smem_a, batch_smem_a(sl.n1d, E, ext));
    *smem_b = std::max(*smem_b, batch_smem_b(sl.n1d, E));
    member_tasks(b, s, seg[ext ? SEG_EXT : SEG_PLAIN]);
    if (tvd) member_tasks(b, s, seg[ext ? SEG_LOW_EXT : SEG_LOW_PLAIN]);
  }
  std::vector<BatchTask> t;
  for (int g = 0; g < NSEG; ++g) {
    std::stable_sort(seg[g].begin(), seg[g].end(), [](const BatchTask& x, const BatchTask& y) {
      auto cost = [](const BatchTask& q) { return q.epb * q.n1d * q.n1d * q.n1d; };
      return cost(x) > cost(y);
    });
    b->seg_off[g] = (int)t.size();
    b->seg_cnt[g] = (int)seg[g].size();
    t.insert(t.end(), seg[g].begin(), seg[g].end());
  }
  if (*smem_a == 0) *smem_a = batch_smem_a(2, 1, false);
  if (*smem_x == 0) *smem_x = batch_smem_a(2, 1, true);
  if (*smem_b == 0) *smem_b = batch_smem_b(2, 1);
  return t;
}

int upload_tasks(p2de_batch* b) {
  size_t sa = 0, sx = 0, sb = 0;
  int cnt_before[NSEG];
  std::memcpy(cnt_before, b->seg_cnt, sizeof cnt_before);
  const bool phi_before = b->phi_min;
  std::vector<BatchTask> t = build_tasks(b, &sa, &sx, &sb);
  b->phi_min = false;
  for (int s = 0; s < b->max_solves; ++s)
    if (b->slots[s].active && (b->slots[s].flags & F_MIN_ENTROPY) && (b->slots[s].flags & F_RELAXED)) b->phi_min = true;
  bool relaunch = sa != b->smem_a || sx != b->smem_x || sb != b->smem_b || b->phi_min != phi_before;
  for (int g = 0; g < NSEG; ++g) relaunch |= (cnt_before[g] > 0) != (b->seg_cnt[g] > 0);
  if (relaunch) {  // launch configuration or the set of launches changes: new capture
    b->smem_a = sa;
    b->smem_x = sx;
    b->smem_b = sb;
    if (b->graph) {
      BCK(cudaStreamSynchronize(b->stream));
      cudaGraphExecDestroy(b->graph);
      b->graph = nullptr;
    }
  }
  if ((int)t.size() > b->task_cap) {
    if (b->d_tasks) {
      BCK(cudaStreamSynchronize(b->stream));
      cudaFree(b->d_tasks);
      b->allocs.erase(std::remove(b->allocs.begin(), b->allocs.end(), (void*)b->d_tasks), b->allocs.end());
      b->d_tasks = nullptr;
    }
    b->task_cap = std::max<int>((int)t.size(), 2 * b->task_cap);
    BCK(balloc(b, &b->d_tasks, (size_t)b->task_cap));
    if (b->graph) {
      cudaGraphExecDestroy(b->graph);
      b->graph = nullptr;
    }
  }
  int nt = (int)t.size();
  if (nt) BCK(cudaMemcpyAsync(b->d_tasks, t.data(), sizeof(BatchTask) * nt, cudaMemcpyHostToDevice, b->stream));
  // task counts: segments 0..3, then segments 0 and 1 together (kernel B)
  int counts[NSEG + 1];
  for (int g = 0; g < NSEG; ++g) counts[g] = b->seg_cnt[g];
  counts[NSEG] = b->seg_cnt[SEG_PLAIN] + b->seg_cnt[SEG_EXT];
  BCK(cudaMemcpyAsync(b->d_ntasks, counts, sizeof counts, cudaMemcpyHostToDevice, b->stream));
  BCK(cudaMemcpyAsync(b->d_active, b->active.data(), b->max_solves, cudaMemcpyHostToDevice, b->stream));
  BCK(cudaStreamSynchronize(b->stream));  // the host vectors above are temporaries
  b->tasks_dirty = false;
  return P2DE_OK;
}

// One step: the step begin, then per stage, in the one-solve path's order, the initial
// minimum of phi (stage 1, relaxed min-entropy members), the low-only pass of the TVD
// members, kernel A over the plain and the EXT members, and kernel B over all of them.
// Passes without tasks are left out (the graph is recaptured when that set changes).
int enqueue_batch_step(p2de_batch* b) {
  BCK(launch_batch_begin(b->d_solves, b->d_active, b->max_solves, b->d_counters, b->stream));
  for (int stage = 1; stage <= 3; ++stage) {
    unsigned* ctr = b->d_counters + kBatchCountersPerStage * (stage - 1);
    if (stage == 1 && b->phi_min) BCK(launch_batch_phi_min(b->d_solves, b->d_active, b->max_solves, b->stream));
    struct Pass {
      int seg, mode;
      bool ext;
    } passes[4] = {{SEG_LOW_PLAIN, BATCH_A_LOW_ONLY, false},
                   {SEG_LOW_EXT, BATCH_A_LOW_ONLY, true},
                   {SEG_PLAIN, BATCH_A_FULL, false},
                   {SEG_EXT, BATCH_A_FULL, true}};
    for (int i = 0; i < 4; ++i) {
      const Pass& q = passes[i];
      if (b->seg_cnt[q.seg] == 0) continue;
      BCK(launch_batch_a(b->mixed, q.ext, q.mode, q.ext ? b->grid_x : b->grid_a, q.ext ? b->smem_x : b->smem_a,
                         b->d_solves, b->d_tasks + b->seg_off[q.seg], b->d_ntasks + q.seg, ctr + i, stage, b->stream));
    }
    BCK(launch_batch_b(b->grid_b, b->smem_b, b->d_solves, b->d_tasks, b->d_ntasks + NSEG, ctr + 4, stage, b->stream));
  }
  return P2DE_OK;
}

// launches of one step (the launch counter)
int step_launch_count(const p2de_batch* b) {
  int n = 1 + (b->phi_min ? 1 : 0);
  for (int g = 0; g < NSEG; ++g) n += 3 * (b->seg_cnt[g] > 0 ? 1 : 0);
  return n + 3;
}

// persistent grids: resident blocks per SM at the current shared memory, times the SMs
int size_grids(p2de_batch* b) {
  int bpa = 0, bpb = 0, bpx = 0, bpb2 = 0;
  BCK(batch_occupancy(b->mixed, false, b->smem_a, b->smem_b, &bpa, &bpb));
  BCK(batch_occupancy(b->mixed, true, b->smem_x, b->smem_b, &bpx, &bpb2));
  if (bpa < 1 || bpb < 1 || bpx < 1) return bfail(b, P2DE_ERR_CUDA, "batched kernels do not fit an SM");
  b->grid_a = b->sms * bpa;
  b->grid_x = b->sms * bpx;
  b->grid_b = b->sms * bpb;
  return P2DE_OK;
}

int build_batch_graph(p2de_batch* b) {
  if (b->graph) return P2DE_OK;
  int rg = size_grids(b);
  if (rg != P2DE_OK) return rg;
  cudaStream_t cap;
  BCK(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
  cudaStream_t user = b->stream;
  b->stream = cap;
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
  int rc = (e == cudaSuccess) ? enqueue_batch_step(b) : P2DE_OK;
  cudaError_t e2 = (e == cudaSuccess) ? cudaStreamEndCapture(cap, &g) : e;
  b->stream = user;
  cudaStreamDestroy(cap);
  if (rc != P2DE_OK) return rc;
  BCK(e);
  BCK(e2);
  BCK(cudaGraphInstantiate(&b->graph, g, 0));
  BCK(cudaGraphDestroy(g));
  return P2DE_OK;
}

}  // namespace

extern "C" {

int p2de_batch_create(int device, int32_t precision, size_t pool_bytes, int32_t max_solves, p2de_batch** out) {
  if (!out || max_solves < 1 || pool_bytes == 0 || precision < 0 || precision > 2) return P2DE_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return P2DE_ERR_NO_DEVICE;
  if (device < 0 || device >= ndev) return P2DE_ERR_INVALID_ARGUMENT;
  p2de_batch* b = new p2de_batch();
  b->device = device;
  b->mixed = precision != P2DE_PRECISION_FP64;
  b->precision = precision;
  b->max_solves = max_solves;
  b->slots.assign(max_solves, Slot{});
  b->active.assign(max_solves, 0);
  auto bail = [&](int code) {
    for (void* p : b->allocs) cudaFree(p);
    b->pool.release();
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return code;
  };
  if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess)
    return bail(P2DE_ERR_CUDA);
  if (b->pool.init(pool_bytes) != cudaSuccess) return bail(P2DE_ERR_OUT_OF_MEMORY);
  if (balloc(b, &b->d_solves, max_solves) != cudaSuccess || balloc(b, &b->d_active, max_solves) != cudaSuccess ||
      balloc(b, &b->d_ntasks, NSEG + 1) != cudaSuccess || balloc(b, &b->d_counters, kBatchCounters + 1) != cudaSuccess ||
      balloc(b, &b->d_scal, (size_t)max_solves * S_NSCAL) != cudaSuccess ||
      balloc(b, &b->d_dtmin, max_solves) != cudaSuccess || balloc(b, &b->d_minrec, (size_t)6 * max_solves) != cudaSuccess ||
      balloc(b, &b->d_status, max_solves) != cudaSuccess || balloc(b, &b->d_work, 8) != cudaSuccess ||
      balloc(b, &b->d_tables, (size_t)kBatchTableGroups * (kMaxN1D - 1)) != cudaSuccess)
    return bail(P2DE_ERR_OUT_OF_MEMORY);
  if (batch_table_group(b, 5e-16) < 0) return bail(P2DE_ERR_CUDA);
  for (int n = 2; n <= kMaxN1D; ++n) {
    StageGeometry geo;
    cudaError_t e = cudaSuccess;
    switch (n) {
      case 2: e = stage_prepare<2>(&geo); break;
      case 3: e = stage_prepare<3>(&geo); break;
      case 4: e = stage_prepare<4>(&geo); break;
      case 5: e = stage_prepare<5>(&geo); break;
      case 6: e = stage_prepare<6>(&geo); break;
    }
    if (e != cudaSuccess) return bail(P2DE_ERR_CUDA);
  }
  if (batch_prepare(b->mixed) != cudaSuccess) return bail(P2DE_ERR_CUDA);
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return bail(P2DE_ERR_CUDA);
  b->sms = prop.multiProcessorCount;
  for (int n = 2; n <= kMaxN1D; ++n) b->epb[n] = batch_elems_per_block(n);
  b->task_cap = 0;
  if (cudaStreamSynchronize(b->stream) != cudaSuccess) return bail(P2DE_ERR_CUDA);
  *out = b;
  return P2DE_OK;
}

int p2de_batch_destroy(p2de_batch* b) {
  if (!b) return P2DE_OK;
  cudaSetDevice(b->device);
  cudaStreamSynchronize(b->stream);
  if (b->graph) cudaGraphExecDestroy(b->graph);
  for (void* p : b->allocs) cudaFree(p);
  b->pool.release();
  cudaStreamDestroy(b->stream);
  delete b;
  return P2DE_OK;
}

int p2de_batch_solve_bytes(const p2de_param* param, int64_t nI, int64_t nS, size_t* bytes) {
  if (!param || !bytes || param->N < 1 || param->N > 5 || param->K < 1) return P2DE_ERR_INVALID_ARGUMENT;
  *bytes = layout_for(*param, nI, nS).total;
  return P2DE_OK;
}

int p2de_batch_add(p2de_batch* b, const p2de_param* p, const p2de_mesh* m, const double* Uq, int32_t* slot_out) {
  if (!b || !Uq || !slot_out) return P2DE_ERR_INVALID_ARGUMENT;
  std::string why;
  int rc = validate_solve(p, m, why);
  if (rc != P2DE_OK) return bfail(b, rc, "%s", why.c_str());
  int slot = -1;
  for (int s = 0; s < b->max_solves; ++s)
    if (!b->slots[s].active) {
      slot = s;
      break;
    }
  if (slot < 0) return bfail(b, P2DE_ERR_BUDGET, "all %d slots in use", b->max_solves);
  Layout lay = layout_for(*p, m->nI, m->nS);
  if (lay.total > b->pool.cap) return bfail(b, P2DE_ERR_BUDGET, "solve needs %zu bytes, pool has %zu", lay.total, b->pool.cap);
  size_t off = 0;
  if (!b->pool.alloc(lay.total, &off)) return bfail(b, P2DE_ERR_BUDGET, "pool full (%zu bytes free)", b->pool.largest_free());
  BCK(cudaSetDevice(b->device));
  char* base = b->pool.base + off;
  const size_t n = p->N + 1, Nq = n * n, Nfp = 4 * n, K = p->K, nfk = Nfp * K;
  std::vector<int32_t> nbr(nfk), bcidx(nfk, 0);
  std::vector<int8_t> bc(nfk, BC_INTERIOR);
  for (size_t i = 0; i < nfk; ++i) nbr[i] = (int32_t)(m->mapP[i] - 1);
  for (int64_t i = 0; i < m->nI; ++i) {
    bc[m->mapI[i] - 1] = BC_INFLOW;
    bcidx[m->mapI[i] - 1] = (int32_t)i;
  }
  for (int64_t i = 0; i < m->nO; ++i) bc[m->mapO[i] - 1] = BC_OUTFLOW;
  for (int64_t i = 0; i < m->nW; ++i) bc[m->mapW[i] - 1] = BC_WALL;
  for (int64_t i = 0; i < m->nS; ++i) {
    bc[m->mapS[i] - 1] = BC_SHOCK;
    bcidx[m->mapS[i] - 1] = (int32_t)i;
  }
  bool aa = true;
  for (size_t k = 0; k < K; ++k)
    if (m->geom[5 * k + 2] != 0.0 || m->geom[5 * k + 3] != 0.0) aa = false;
  auto up = [&](size_t o, const void* src, size_t bytes) {
    return cudaMemcpyAsync(base + o, src, bytes, cudaMemcpyHostToDevice, b->stream);
  };
  BCK(up(lay.Uq, Uq, 8 * 4 * Nq * K));
  BCK(up(lay.geom, m->geom, 8 * 5 * K));
  BCK(launch_geom_table((const double*)(base + lay.geom), (int)K, (double*)(base + lay.geomx), b->stream));
  BCK(up(lay.nbr, nbr.data(), 4 * nfk));
  BCK(up(lay.bcidx, bcidx.data(), 4 * nfk));
  BCK(up(lay.bc, bc.data(), nfk));
  if (m->nI > 0) BCK(up(lay.Ival, m->Ival, 8 * 4 * m->nI));
  if (m->nS > 0) BCK(up(lay.xyS, m->xyS, 8 * 2 * m->nS));
  StageArgs a{};
  a.K = p->K;
  a.nstage = 1;
  const int f = member_flags(*p, aa, b->precision);
  a.flags = f;
  set_shock_capture(a, p->N, p->shock_capture_a, p->shock_capture_c);
  set_bound_constants(a, p->N, p->t0, p->POSTOL, p->bound_beta);
  a.eta = p->eta;
  a.rhoL = (double*)(base + lay.rhoL);
  a.Lelem = (double*)(base + lay.Lelem);
  a.phimin = (double*)(base + lay.phimin);
  const int tg = batch_table_group(b, p->ZEROTOL);
  if (tg < 0)
    return bfail(b, P2DE_ERR_UNSUPPORTED, "more than %d distinct ZEROTOL values in one batch", kBatchTableGroups);
  a.ops = b->d_tables + (size_t)tg * (kMaxN1D - 1) + (n - 2);
  a.Uq = (double*)(base + lay.Uq);
  a.resW = (double*)(base + lay.resW);
  a.geom = (const double*)(base + lay.geom);
  a.geomx = (const double*)(base + lay.geomx);
  a.nbr = (const int32_t*)(base + lay.nbr);
  a.bc = (const int8_t*)(base + lay.bc);
  a.bcidx = (const int32_t*)(base + lay.bcidx);
  a.Ival = (const double*)(base + lay.Ival);
  a.xyS = (const double*)(base + lay.xyS);
  a.shock_x0 = m->shock_x0;
  a.shock_inv_slope = m->shock_inv_slope;
  a.shock_speed = m->shock_speed;
  for (int c = 0; c < 4; ++c) {
    a.shock_post[c] = m->shock_post[c];
    a.shock_pre[c] = m->shock_pre[c];
  }
  a.gamma = p->gamma;
  a.gm1 = p->gamma - 1.0;
  a.CFL = p->CFL;
  a.dt0 = p->dt0;
  a.T = p->T;
  a.zeta = p->zeta;
  a.ZEROTOL = p->ZEROTOL;
  a.rhsL = (double*)(base + lay.rhsL);
  a.rhsH = (double*)(base + lay.rhsH);
  a.rhsU = (double*)(base + lay.rhsU);
  a.rhsxyL = a.rhsxyH = a.BFL = a.BFH = nullptr;
  a.fbar = (double*)(base + lay.fbar);
  a.Lpre = (double*)(base + lay.Lpre);
  a.Lfin = (double*)(base + lay.Lfin);
  a.scal = b->d_scal + (size_t)slot * S_NSCAL;
  a.dtmin_bits = b->d_dtmin + slot;
  a.minrec = b->d_minrec + 6 * (size_t)slot;
  a.status = b->d_status + slot;
  a.counters = b->d_work;
  double sc[S_NSCAL] = {0};
  sc[S_T] = p->t0;
  int zero = 0;
  BCK(cudaMemcpyAsync(a.scal, sc, sizeof sc, cudaMemcpyHostToDevice, b->stream));
  BCK(cudaMemcpyAsync(a.status, &zero, sizeof zero, cudaMemcpyHostToDevice, b->stream));
  BCK(cudaMemcpyAsync(b->d_solves + slot, &a, sizeof a, cudaMemcpyHostToDevice, b->stream));
  BCK(cudaStreamSynchronize(b->stream));  // host buffers above are temporaries
  Slot& sl = b->slots[slot];
  sl.active = true;
  sl.prm = *p;
  sl.n1d = (int)n;
  sl.flags = f;
  sl.off = off;
  sl.lay = lay;
  b->active[slot] = 1;
  b->tasks_dirty = true;
  *slot_out = slot;
  return P2DE_OK;
}

int p2de_batch_remove(p2de_batch* b, int32_t slot) {
  if (!b || slot < 0 || slot >= b->max_solves || !b->slots[slot].active) return P2DE_ERR_NOT_FOUND;
  BCK(cudaSetDevice(b->device));
  BCK(cudaStreamSynchronize(b->stream));
  b->pool.release_block(b->slots[slot].off);
  b->slots[slot].active = false;
  b->active[slot] = 0;
  b->tasks_dirty = true;
  return P2DE_OK;
}

int p2de_batch_step(p2de_batch* b, int64_t nsteps) {
  if (!b || nsteps < 0) return P2DE_ERR_INVALID_ARGUMENT;
  BCK(cudaSetDevice(b->device));
  if (b->tasks_dirty) {
    int rc = upload_tasks(b);
    if (rc != P2DE_OK) return rc;
  }
  int rc = build_batch_graph(b);
  if (rc != P2DE_OK) return rc;
  for (int64_t i = 0; i < nsteps; ++i) {
    BCK(cudaGraphLaunch(b->graph, b->stream));
    b->launches += step_launch_count(b);
  }
  BCK(cudaStreamSynchronize(b->stream));
  return P2DE_OK;
}

int p2de_batch_set_elements_per_block(p2de_batch* b, int32_t N, int32_t epb) {
  if (!b || N < 1 || N + 1 > kMaxN1D) return P2DE_ERR_INVALID_ARGUMENT;
  const int emax = batch_elems_per_block_max(N + 1);
  if (epb < 1 || epb > emax)
    return bfail(b, P2DE_ERR_INVALID_ARGUMENT, "elements per block %d outside 1..%d", epb, emax);
  if (b->epb[N + 1] != epb) {
    b->epb[N + 1] = epb;
    b->tasks_dirty = true;
  }
  return P2DE_OK;
}

int p2de_batch_set_layout(p2de_batch* b, int32_t N, int32_t layout) {
  if (!b || N < 1 || N + 1 > kMaxN1D) return P2DE_ERR_INVALID_ARGUMENT;
  if (layout != P2DE_LAYOUT_FLAT && layout != P2DE_LAYOUT_LINES_PER_WARP)
    return bfail(b, P2DE_ERR_INVALID_ARGUMENT, "layout %d", layout);
  if (b->layout[N + 1] != layout) {
    b->layout[N + 1] = layout;
    b->tasks_dirty = true;
  }
  return P2DE_OK;
}

int p2de_batch_get_layout(p2de_batch* b, int32_t N, int32_t* layout) {
  if (!b || !layout || N < 1 || N + 1 > kMaxN1D) return P2DE_ERR_INVALID_ARGUMENT;
  *layout = b->layout[N + 1];
  return P2DE_OK;
}

int p2de_batch_get_elements_per_block(p2de_batch* b, int32_t N, int32_t* epb, int32_t* epb_max) {
  if (!b || N < 1 || N + 1 > kMaxN1D) return P2DE_ERR_INVALID_ARGUMENT;
  if (epb) *epb = b->epb[N + 1];
  if (epb_max) *epb_max = batch_elems_per_block_max(N + 1);
  return P2DE_OK;
}

// For each degree present in the batch, times batched stage kernel A (stage 2 flags;
// it writes only stage scratch, so no solve's state changes) over that degree's
// solves for each candidate elements-per-block, and keeps the fastest.
int p2de_batch_autotune(p2de_batch* b, int32_t best_epb[5]) {
  if (!b) return P2DE_ERR_INVALID_ARGUMENT;
  BCK(cudaSetDevice(b->device));
  BCK(cudaStreamSynchronize(b->stream));
  if (best_epb)
    for (int i = 0; i < 5; ++i) best_epb[i] = 0;
  std::vector<double> keep((size_t)b->max_solves * S_NSCAL);
  BCK(cudaMemcpyAsync(keep.data(), b->d_scal, sizeof(double) * keep.size(), cudaMemcpyDeviceToHost, b->stream));
  BCK(cudaStreamSynchronize(b->stream));
  std::vector<double> sc = keep;
  int64_t ksum = 0;
  for (int s = 0; s < b->max_solves; ++s) {
    const Slot& sl = b->slots[s];
    if (!sl.active) continue;
    ksum += sl.prm.K;
    double* q = &sc[(size_t)s * S_NSCAL];
    q[S_DONE] = 0.0;
    if (!(q[S_DT_LIM] > 0.0)) q[S_DT_LIM] = std::fmin(sl.prm.CFL * sl.prm.dt0, sl.prm.T - sl.prm.t0);
  }
  if (ksum == 0) return P2DE_OK;
  if (ksum > b->task_cap) {  // room for one task per element
    if (b->d_tasks) {
      cudaFree(b->d_tasks);
      b->allocs.erase(std::remove(b->allocs.begin(), b->allocs.end(), (void*)b->d_tasks), b->allocs.end());
      b->d_tasks = nullptr;
    }
    b->task_cap = (int)ksum;
    BCK(balloc(b, &b->d_tasks, (size_t)b->task_cap));
  }
  if (b->graph) {  // the task list is rewritten below
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
  b->tasks_dirty = true;
  BCK(cudaMemcpyAsync(b->d_scal, sc.data(), sizeof(double) * sc.size(), cudaMemcpyHostToDevice, b->stream));
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  unsigned* counter = b->d_counters + kBatchCounters;  // the spare counter
  // the timings; whatever they return, the events go and the scalars come back below
  auto timings = [&]() -> int {
  BCK(cudaEventCreate(&e0));
  BCK(cudaEventCreate(&e1));
  for (int n1d = 2; n1d <= kMaxN1D; ++n1d) {
    bool present = false;
    for (int s = 0; s < b->max_solves; ++s) present |= b->slots[s].active && b->slots[s].n1d == n1d;
    if (!present) continue;
    const int emax = batch_elems_per_block_max(n1d), edef = batch_elems_per_block(n1d);
    int best = b->epb[n1d], best_layout = b->layout[n1d];
    double bms = 1e30;
    for (int lay : {(int)P2DE_LAYOUT_FLAT, (int)P2DE_LAYOUT_LINES_PER_WARP})
    for (int e : {1, 2, 3, 4, 6, 8, 12, 16, 24, 32, edef}) {
      if (e > emax) continue;
      // this degree's members, plain and EXT instantiation, full pass at stage 2
      std::vector<BatchTask> t[2];
      for (int s = 0; s < b->max_solves; ++s) {
        const Slot& sl = b->slots[s];
        if (!sl.active || sl.n1d != n1d) continue;
        const int x = (sl.flags & kExtFlags) ? 1 : 0;
        for (int k0 = 0; k0 < sl.prm.K; k0 += e) t[x].push_back(BatchTask{s, k0, n1d, e, lay});
      }
      int grid[2] = {0, 0}, nt[2] = {(int)t[0].size(), (int)t[1].size()};
      size_t sm[2] = {batch_smem_a(n1d, e, false), batch_smem_a(n1d, e, true)};
      bool fits = true;
      for (int x = 0; x < 2; ++x) {
        if (!nt[x]) continue;
        int bpa = 0, bpb = 0;
        cudaError_t ce = batch_occupancy(b->mixed, x == 1, sm[x], batch_smem_b(n1d, e), &bpa, &bpb);
        if (ce != cudaSuccess || bpa < 1) fits = false;
        grid[x] = std::min(b->sms * bpa, nt[x]);
      }
      if (!fits) continue;
      std::vector<BatchTask> all = t[0];
      all.insert(all.end(), t[1].begin(), t[1].end());
      BCK(cudaMemcpyAsync(b->d_tasks, all.data(), sizeof(BatchTask) * all.size(), cudaMemcpyHostToDevice, b->stream));
      BCK(cudaMemcpyAsync(b->d_ntasks, nt, sizeof nt, cudaMemcpyHostToDevice, b->stream));
      float tot = 0.f;
      for (int rep = 0; rep < 4; ++rep) {
        BCK(cudaEventRecord(e0, b->stream));
        for (int x = 0; x < 2; ++x) {
          if (!nt[x]) continue;
          BCK(cudaMemsetAsync(counter, 0, sizeof(unsigned), b->stream));
          BCK(launch_batch_a(b->mixed, x == 1, BATCH_A_FULL, grid[x], sm[x], b->d_solves, b->d_tasks + (x ? nt[0] : 0),
                             b->d_ntasks + x, counter, 2, b->stream));
          b->launches += 1;
        }
        BCK(cudaEventRecord(e1, b->stream));
        BCK(cudaEventSynchronize(e1));
        float ms;
        BCK(cudaEventElapsedTime(&ms, e0, e1));
        if (rep > 0) tot += ms;  // first launch warms up
      }
      if (tot / 3.0 < bms) {
        bms = tot / 3.0;
        best = e;
        best_layout = lay;
      }
    }
    b->epb[n1d] = best;
    b->layout[n1d] = best_layout;
    if (best_epb) best_epb[n1d - 2] = best;
  }
  return P2DE_OK;
  };
  const int rc = timings();
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  BCK(cudaMemcpyAsync(b->d_scal, keep.data(), sizeof(double) * keep.size(), cudaMemcpyHostToDevice, b->stream));
  BCK(cudaStreamSynchronize(b->stream));  // the host vectors above are temporaries
  return rc;
}

int p2de_batch_state(p2de_batch* b, int32_t slot, double* t, double* dt, int64_t* steps, int32_t* done,
                     int32_t* status) {
  if (!b || slot < 0 || slot >= b->max_solves || !b->slots[slot].active) return P2DE_ERR_NOT_FOUND;
  BCK(cudaSetDevice(b->device));
  double sc[S_NSCAL];
  int st = 0;
  BCK(cudaMemcpyAsync(sc, b->d_scal + (size_t)slot * S_NSCAL, sizeof sc, cudaMemcpyDeviceToHost, b->stream));
  BCK(cudaMemcpyAsync(&st, b->d_status + slot, sizeof st, cudaMemcpyDeviceToHost, b->stream));
  BCK(cudaStreamSynchronize(b->stream));
  if (t) *t = sc[S_T];
  if (dt) *dt = sc[S_DT];
  if (steps) *steps = (int64_t)sc[S_STEPS];
  if (done) *done = (!(sc[S_T] < b->slots[slot].prm.T) || st != 0) ? 1 : 0;
  if (status) *status = st;
  return P2DE_OK;
}

// All slots' (t, steps, done, status) in one transfer; out is max_solves x 4.
int p2de_batch_states(p2de_batch* b, double* out) {
  if (!b || !out) return P2DE_ERR_INVALID_ARGUMENT;
  BCK(cudaSetDevice(b->device));
  std::vector<double> sc((size_t)b->max_solves * S_NSCAL);
  std::vector<int> st(b->max_solves);
  BCK(cudaMemcpyAsync(sc.data(), b->d_scal, sizeof(double) * sc.size(), cudaMemcpyDeviceToHost, b->stream));
  BCK(cudaMemcpyAsync(st.data(), b->d_status, sizeof(int) * st.size(), cudaMemcpyDeviceToHost, b->stream));
  BCK(cudaStreamSynchronize(b->stream));
  for (int s = 0; s < b->max_solves; ++s) {
    double t = sc[(size_t)s * S_NSCAL + S_T];
    bool act = b->slots[s].active;
    out[4 * s + 0] = t;
    out[4 * s + 1] = sc[(size_t)s * S_NSCAL + S_STEPS];
    out[4 * s + 2] = act && (!(t < b->slots[s].prm.T) || st[s] != 0) ? 1.0 : 0.0;
    out[4 * s + 3] = act ? (double)st[s] : -1.0;
  }
  return P2DE_OK;
}

int p2de_batch_get_Uq(p2de_batch* b, int32_t slot, double* Uq) {
  if (!b || !Uq || slot < 0 || slot >= b->max_solves || !b->slots[slot].active) return P2DE_ERR_NOT_FOUND;
  BCK(cudaSetDevice(b->device));
  const Slot& sl = b->slots[slot];
  size_t bytes = 8 * 4 * (size_t)sl.n1d * sl.n1d * sl.prm.K;
  BCK(cudaMemcpyAsync(Uq, b->pool.base + sl.off + sl.lay.Uq, bytes, cudaMemcpyDeviceToHost, b->stream));
  BCK(cudaStreamSynchronize(b->stream));
  return P2DE_OK;
}

int p2de_batch_memory(p2de_batch* b, size_t* used, size_t* capacity) {
  if (!b) return P2DE_ERR_INVALID_ARGUMENT;
  if (used) *used = b->pool.in_use;
  if (capacity) *capacity = b->pool.cap;
  return P2DE_OK;
}

int p2de_batch_launch_count(p2de_batch* b, int64_t* count) {
  if (!b || !count) return P2DE_ERR_INVALID_ARGUMENT;
  *count = b->launches;
  return P2DE_OK;
}

int p2de_batch_last_error(p2de_batch* b, char* buf, size_t len) {
  if (!b || !buf || len == 0) return P2DE_ERR_INVALID_ARGUMENT;
  std::snprintf(buf, len, "%s", b->err.c_str());
  return P2DE_OK;
}

}  // extern "C"

// =====================================================================================
// Continuous-batching server
// =====================================================================================
namespace {

struct Request {
  int64_t id = 0;
  p2de_param prm{};
  std::vector<double> geom, Ival, xyS, Uq;
  std::vector<int64_t> mapP, mapI, mapO, mapW, mapS;
  double shock[11] = {0};
  size_t bytes = 0;
  int state = 0;  // 0 queued, 1 running, 2 done, 3 failed
  int slot = -1;
  double t_submit = 0, t_admit = 0, t_done = 0, t_final = 0;
  int64_t steps = 0;
  int status = 0;
};

p2de_mesh mesh_of(const Request& r) {
  p2de_mesh m{};
  m.geom = r.geom.data();
  m.mapP = r.mapP.data();
  m.mapI = r.mapI.data();
  m.nI = (int64_t)r.mapI.size();
  m.Ival = r.Ival.data();
  m.mapO = r.mapO.data();
  m.nO = (int64_t)r.mapO.size();
  m.mapW = r.mapW.data();
  m.nW = (int64_t)r.mapW.size();
  m.mapS = r.mapS.data();
  m.nS = (int64_t)r.mapS.size();
  m.xyS = r.xyS.data();
  m.shock_x0 = r.shock[0];
  m.shock_inv_slope = r.shock[1];
  m.shock_speed = r.shock[2];
  for (int c = 0; c < 4; ++c) {
    m.shock_post[c] = r.shock[3 + c];
    m.shock_pre[c] = r.shock[7 + c];
  }
  return m;
}

}  // namespace

struct p2de_server {
  p2de_batch* batch = nullptr;
  int max_active = 0;
  int steps_per_tick = 1;
  std::mutex mu;
  std::condition_variable cv;
  std::deque<int64_t> queue;
  std::unordered_map<int64_t, Request> reqs;
  std::unordered_map<int, int64_t> slot_req;
  std::thread worker;
  bool stop = false;
  int64_t next_id = 1;
  int64_t completed = 0, failed = 0, ticks = 0;
  double busy_s = 0.0;
  std::string err;
};

namespace {

void server_loop(p2de_server* sv) {
  cudaSetDevice(sv->batch->device);
  std::vector<double> states((size_t)sv->batch->max_solves * 4);
  for (;;) {
    // admit queued requests that fit, first come first served, skipping ones that do not fit yet
    std::vector<int64_t> admit;
    {
      std::unique_lock<std::mutex> lk(sv->mu);
      sv->cv.wait(lk, [&] { return sv->stop || !sv->queue.empty() || !sv->slot_req.empty(); });
      if (sv->stop) return;
      int active = (int)sv->slot_req.size();
      size_t room = sv->batch->pool.cap - sv->batch->pool.in_use;
      for (auto it = sv->queue.begin(); it != sv->queue.end() && active + (int)admit.size() < sv->max_active;) {
        Request& r = sv->reqs[*it];
        if (r.bytes <= room) {
          admit.push_back(*it);
          room -= r.bytes;
          it = sv->queue.erase(it);
        } else {
          ++it;
        }
      }
    }
    for (int64_t id : admit) {
      Request* r;
      {
        std::lock_guard<std::mutex> lk(sv->mu);
        r = &sv->reqs[id];
      }
      p2de_mesh m = mesh_of(*r);
      int32_t slot = -1;
      int rc = p2de_batch_add(sv->batch, &r->prm, &m, r->Uq.data(), &slot);
      std::lock_guard<std::mutex> lk(sv->mu);
      if (rc == P2DE_OK) {
        r->state = 1;
        r->slot = slot;
        r->t_admit = now_s();
        sv->slot_req[slot] = id;
      } else if (rc == P2DE_ERR_BUDGET) {
        sv->queue.push_front(id);  // pool fragmentation: try again after a retirement
      } else {
        r->state = 3;
        r->status = rc;
        r->t_done = now_s();
        sv->failed++;
        sv->cv.notify_all();
      }
    }
    bool any;
    {
      std::lock_guard<std::mutex> lk(sv->mu);
      any = !sv->slot_req.empty();
    }
    if (!any) continue;
    double t0 = now_s();
    int rc = p2de_batch_step(sv->batch, sv->steps_per_tick);
    if (rc == P2DE_OK) rc = p2de_batch_states(sv->batch, states.data());
    sv->busy_s += now_s() - t0;
    sv->ticks++;
    // retire finished solves
    std::vector<std::pair<int, int64_t>> done;
    {
      std::lock_guard<std::mutex> lk(sv->mu);
      for (auto& kv : sv->slot_req)
        if (rc != P2DE_OK || states[4 * kv.first + 2] != 0.0) done.push_back({kv.first, kv.second});
    }
    for (auto& d : done) {
      Request* r;
      {
        std::lock_guard<std::mutex> lk(sv->mu);
        r = &sv->reqs[d.second];
      }
      int rc2 = p2de_batch_get_Uq(sv->batch, d.first, r->Uq.data());
      double tt = states[4 * d.first], steps = states[4 * d.first + 1];
      int st = (int)states[4 * d.first + 3];
      p2de_batch_remove(sv->batch, d.first);
      std::lock_guard<std::mutex> lk(sv->mu);
      r->t_done = now_s();
      r->t_final = tt;
      r->steps = (int64_t)steps;
      r->status = st;
      bool ok = rc == P2DE_OK && rc2 == P2DE_OK && st == 0;
      r->state = ok ? 2 : 3;
      if (ok)
        sv->completed++;
      else
        sv->failed++;
      sv->slot_req.erase(d.first);
      sv->cv.notify_all();
    }
  }
}

}  // namespace

extern "C" {

int p2de_server_create(int device, int32_t precision, size_t hbm_budget_bytes, int32_t max_active,
                       int32_t steps_per_tick, p2de_server** out) {
  if (!out || max_active < 1 || steps_per_tick < 1) return P2DE_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  p2de_batch* b = nullptr;
  int rc = p2de_batch_create(device, precision, hbm_budget_bytes, max_active, &b);
  if (rc != P2DE_OK) return rc;
  p2de_server* sv = new p2de_server();
  sv->batch = b;
  sv->max_active = max_active;
  sv->steps_per_tick = steps_per_tick;
  sv->worker = std::thread(server_loop, sv);
  *out = sv;
  return P2DE_OK;
}

int p2de_server_submit(p2de_server* sv, const p2de_param* p, const p2de_mesh* m, const double* Uq, int64_t* id) {
  if (!sv || !Uq || !id) return P2DE_ERR_INVALID_ARGUMENT;
  std::string why;
  int rc = validate_solve(p, m, why);
  if (rc != P2DE_OK) {
    std::lock_guard<std::mutex> lk(sv->mu);
    sv->err = why;
    return rc;
  }
  Request r;
  r.prm = *p;
  const size_t n = p->N + 1, Nq = n * n, K = p->K, nfk = 4 * n * K;
  r.geom.assign(m->geom, m->geom + 5 * K);
  r.mapP.assign(m->mapP, m->mapP + nfk);
  if (m->nI > 0) {
    r.mapI.assign(m->mapI, m->mapI + m->nI);
    r.Ival.assign(m->Ival, m->Ival + 4 * m->nI);
  }
  if (m->nO > 0) r.mapO.assign(m->mapO, m->mapO + m->nO);
  if (m->nW > 0) r.mapW.assign(m->mapW, m->mapW + m->nW);
  if (m->nS > 0) {
    r.mapS.assign(m->mapS, m->mapS + m->nS);
    r.xyS.assign(m->xyS, m->xyS + 2 * m->nS);
  }
  r.shock[0] = m->shock_x0;
  r.shock[1] = m->shock_inv_slope;
  r.shock[2] = m->shock_speed;
  for (int c = 0; c < 4; ++c) {
    r.shock[3 + c] = m->shock_post[c];
    r.shock[7 + c] = m->shock_pre[c];
  }
  r.Uq.assign(Uq, Uq + 4 * Nq * K);
  r.bytes = layout_for(*p, m->nI, m->nS).total;
  if (r.bytes > sv->batch->pool.cap) {
    std::lock_guard<std::mutex> lk(sv->mu);
    sv->err = "request larger than the HBM budget";
    return P2DE_ERR_BUDGET;
  }
  r.t_submit = now_s();
  std::lock_guard<std::mutex> lk(sv->mu);
  r.id = sv->next_id++;
  *id = r.id;
  sv->reqs.emplace(r.id, std::move(r));
  sv->queue.push_back(*id);
  sv->cv.notify_all();
  return P2DE_OK;
}

int p2de_server_poll(p2de_server* sv, int64_t id, int32_t* state, double* latency_s, double* t_final, int64_t* steps) {
  if (!sv) return P2DE_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(sv->mu);
  auto it = sv->reqs.find(id);
  if (it == sv->reqs.end()) return P2DE_ERR_NOT_FOUND;
  const Request& r = it->second;
  if (state) *state = r.state;
  if (latency_s) *latency_s = r.state >= 2 ? r.t_done - r.t_submit : -1.0;
  if (t_final) *t_final = r.t_final;
  if (steps) *steps = r.steps;
  return P2DE_OK;
}

// Blocks until the request is done or failed, or until timeout_s passes.
int p2de_server_wait(p2de_server* sv, int64_t id, double timeout_s, int32_t* state) {
  if (!sv) return P2DE_ERR_INVALID_ARGUMENT;
  std::unique_lock<std::mutex> lk(sv->mu);
  auto deadline = std::chrono::steady_clock::now() + std::chrono::duration<double>(timeout_s);
  for (;;) {
    auto it = sv->reqs.find(id);
    if (it == sv->reqs.end()) return P2DE_ERR_NOT_FOUND;
    if (it->second.state >= 2) {
      if (state) *state = it->second.state;
      return P2DE_OK;
    }
    if (sv->cv.wait_until(lk, deadline) == std::cv_status::timeout) {
      if (state) *state = it->second.state;
      return P2DE_OK;
    }
  }
}

// Copies the final state of a finished request and forgets the request.
int p2de_server_result(p2de_server* sv, int64_t id, double* Uq) {
  if (!sv || !Uq) return P2DE_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(sv->mu);
  auto it = sv->reqs.find(id);
  if (it == sv->reqs.end()) return P2DE_ERR_NOT_FOUND;
  if (it->second.state < 2) return P2DE_ERR_INVALID_ARGUMENT;
  std::memcpy(Uq, it->second.Uq.data(), sizeof(double) * it->second.Uq.size());
  int st = it->second.state;
  sv->reqs.erase(it);
  return st == 2 ? P2DE_OK : P2DE_ERR_NOT_POSITIVE;
}

// stats: completed, failed, active, queued, pool bytes in use, pool capacity, ticks, busy seconds
int p2de_server_stats(p2de_server* sv, double out[8]) {
  if (!sv || !out) return P2DE_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(sv->mu);
  out[0] = (double)sv->completed;
  out[1] = (double)sv->failed;
  out[2] = (double)sv->slot_req.size();
  out[3] = (double)sv->queue.size();
  out[4] = (double)sv->batch->pool.in_use;
  out[5] = (double)sv->batch->pool.cap;
  out[6] = (double)sv->ticks;
  out[7] = sv->busy_s;
  return P2DE_OK;
}

int p2de_server_destroy(p2de_server* sv) {
  if (!sv) return P2DE_OK;
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    sv->stop = true;
    sv->cv.notify_all();
  }
  if (sv->worker.joinable()) sv->worker.join();
  p2de_batch_destroy(sv->batch);
  delete sv;
  return P2DE_OK;
}

}  // extern "C"
