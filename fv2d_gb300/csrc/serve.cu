// serve.cu -- the batched FP32 service (include/fv2d_serve.h).
//
// Host side: a worker thread owns the GPU stream.  Between graph replays it
//   1. admits queued requests while the HBM budget allows (state buffers come
//      from a chunked arena, so admission does not call cudaMalloc once the
//      arena has grown to the working-set size),
//   2. initialises them on the device (initial condition in binary64 ->
//      binary32 state with its ghost ring, first dt, conservation sums),
//   3. rebuilds the per-bucket (simulation, tile) work lists,
//   4. replays a CUDA graph of K steps (K sized to ~3 ms of work), where each
//      step is one persistent-kernel launch per non-empty grid-size bucket,
//   5. reads the simulation table back and retires finished simulations
//      (final conservation sums, state copied to host memory, arena freed).
#include <cudaTypedefs.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/fv2d_serve.h"
#include "arena.hpp"
#include "batch_common.cuh"
#include "ic.h"
#include "physics.cuh"
#include "problems.h"
#include "schedule.hpp"
#include "nvtx_range.h"

namespace fv2d {
int batch_num_cfgs();
void batch_cfg_info(int i, int *tx, int *ty, int *nt, int *staging, size_t *smem, const char **name, int *ext);
cudaError_t batch_setup(int i, int *ctas_per_sm);
cudaError_t batch_launch(int i, int grid, cudaStream_t s, const BatchArgs &a);
}  // namespace fv2d

using namespace fv2d;

namespace {

constexpr int kBuckets = 4;
// Work lists, kernel launches and graph branches are per lane: a grid-size
// bucket of one kernel family (lanes 0-3 the plain family, 4-7 the diffusive
// one, 8-11 the extended one).
constexpr int kLanes = kFamilies * kBuckets;
int num_cfgs() { return batch_num_cfgs(); }
constexpr int kConsBlocks = 64;
constexpr int kMinSide = 16, kMaxSide = 8192;  // accepted Nx, Ny
static_assert(offsetof(SimDev, band) == offsetof(SimDev, nty) + sizeof(int), "nty and band are updated by one copy");

// Grid-size bucket of an Nx x Ny grid, by its cell count (the side of the
// square with as many cells: < 128, < 256, < 512, larger).
int bucket_of(int Nx, int Ny) {
  const double c = (double)Nx * Ny;
  return c < 128.0 * 128 ? 0 : (c < 256.0 * 256 ? 1 : (c < 512.0 * 512 ? 2 : 3));
}
// kernel families configuration c runs (bit FAM_*)
int cfg_fams(int c) {
  int f = 0;
  batch_cfg_info(c, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, &f);
  return f;
}

// ---------------------------------------------------------------- kernels
// Initial state of one simulation: every padded cell (ghosts included) takes
// the binary64 initial condition of its source cell (BoundaryConditions.h
// maps), converted to conservative variables and stored in binary32 as the
// offset from the background (bg_r, 0, 0, bg_e).
__global__ void ic_kernel(fv2d_params p, int problem, float *U, long long plane, int pitch, int Nx, int Ny,
                          float bg_r, float bg_e) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int W = Nx + 4;
  if (idx >= (long long)W * (Ny + 4)) return;
  const int py = (int)(idx / W), px = (int)(idx % W);
  int sx = px - 2, sy = py - 2;
  bool nx = false, ny = false;
  if (sx < 0 || sx >= Nx) sx = ghost_source(sx, Nx, p.boundary_x, &nx);
  if (sy < 0 || sy >= Ny) sy = ghost_source(sy, Ny, p.boundary_y, &ny);
  double q[4];
  init_cell(p, problem, sx, sy, q);
  if (nx) q[1] = -q[1];
  if (ny) q[2] = -q[2];
  const Gas<double> g{p.gamma0, p.gamma0 - 1.0, 1.0 / (p.gamma0 - 1.0), 0.0};
  const S4<double> u = prim_to_cons(S4<double>{q[0], q[1], q[2], q[3]}, g);
  const long long o = (long long)py * pitch + px;
  U[o] = (float)(u.r - (double)bg_r);
  U[plane + o] = (float)u.u;
  U[2 * plane + o] = (float)u.v;
  U[3 * plane + o] = (float)(u.p - (double)bg_e);
}

// Per-row table of simulation `slot`: the row's gravity (Gravity.h:15-37,
// narrowed to float like :16, 39) and face conductivities
// (ThermalConduction.h:9-26, 46-53: the neighbour conductivities are taken at
// the physical coordinates converted to int, as the reference calls them).
__device__ double row_kappa(const fv2d_params &p, int jj) {  // padded row jj
  if (p.thermal_conductivity_mode == FV2D_TCM_B02) {
    const double dy = (p.ymax - p.ymin) / p.Ny;
    const double y = p.ymin + (jj - p.Nghosts + 0.5) * dy;
    const double tr = (tanh((y - p.b02_ymid) / p.b02_thickness) + 1.0) * 0.5;
    return p.kappa * (p.b02_kappa1 * (1.0 - tr) + p.b02_kappa2 * tr);
  }
  return p.kappa;
}
__global__ void rows_kernel(fv2d_params p, float *rows) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= p.Ny) return;
  const double dy = (p.ymax - p.ymin) / p.Ny;
  const double y = p.ymin + ((double)j + 0.5) * dy;
  float *r = rows + (size_t)j * kRowStride;
  r[ROW_G] = (float)(p.hot_bubble_g0 * sin(y * M_PI * 2.0 / p.ymax));
  const double kC = row_kappa(p, j + p.Nghosts);
  r[ROW_KL] = (float)(0.5 * (kC + row_kappa(p, (int)y)));
  r[ROW_KR] = (float)(0.5 * (kC + row_kappa(p, (int)y)));
  r[ROW_KU] = (float)(0.5 * (kC + row_kappa(p, (int)(y - dy))));
  r[ROW_KD] = (float)(0.5 * (kC + row_kappa(p, (int)(y + dy))));
  r[5] = r[6] = r[7] = 0.f;
}

// Inverse hyperbolic dt of the current state of simulation `slot` (same
// per-cell expression as the step epilogue), max into acc_bits.
__global__ void first_dt_kernel(SimDev *sims, int slot) {
  const SimDev &S = sims[slot];
  const int Nx = S.Nx;
  const float *U = S.U[S.cur];
  float m = 0.f;
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < (long long)Nx * S.Ny;
       c += (long long)gridDim.x * blockDim.x) {
    const int j = (int)(c / Nx), i = (int)(c % Nx);
    const long long g = (long long)(j + 2) * S.pitch + (i + 2);
    float r = U[g] + S.bg_r, u = U[S.plane + g] / r, v = U[2 * S.plane + g] / r;
    float p = pressure_of(U[3 * S.plane + g], S.bg_e, r, u, v, S.gm1, S.lowmach);
    if (r < 0.f) r = 1e-8f;
    if (p < 0.f) p = 1e-8f;
    const float cs = sqrtf(p * S.gamma / r);
    const float ih = (cs + fabsf(u)) * S.inv_dx + (cs + fabsf(v)) * S.inv_dy;
    if (ih > m) m = ih;
  }
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(&sims[slot].acc_bits, __float_as_uint(m));
}

__global__ void first_dt_finish(SimDev *sims, int slot) {
  SimDev &S = sims[slot];
  double m = (double)__uint_as_float(S.acc_bits);
  if (m < S.inv_tc) m = S.inv_tc;
  if (m < S.inv_visc) m = S.inv_visc;
  S.dt = S.cfl / m;
  S.acc_bits = 0u;
  if (!(S.dt > 0.0) || isinf(S.dt)) S.status = SIM_FAILED;
  if (S.max_steps <= 0 || !(S.t + S.eps < S.tend)) S.status = SIM_DONE;
}

// Compensated (Neumaier) binary64 partial sums of the four conserved fields
// of simulation `slot`; out[block][field][sum, compensation].
__device__ __forceinline__ void neumaier_add(double &s, double &c, double x) {
  const double t = s + x;
  c += (fabs(s) >= fabs(x)) ? (s - t) + x : (x - t) + s;
  s = t;
}
__global__ void __launch_bounds__(256) cons_kernel(const SimDev *sims, int slot, double *out) {
  const SimDev &S = sims[slot];
  const int Nx = S.Nx;
  const float *U = S.U[S.cur];
  const double bg[4] = {(double)S.bg_r, 0.0, 0.0, (double)S.bg_e};
  double s[4] = {0, 0, 0, 0}, c[4] = {0, 0, 0, 0};
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < (long long)Nx * S.Ny;
       k += (long long)gridDim.x * blockDim.x) {
    const int j = (int)(k / Nx), i = (int)(k % Nx);
    const long long g = (long long)(j + 2) * S.pitch + (i + 2);
    for (int f = 0; f < 4; ++f) neumaier_add(s[f], c[f], (double)U[f * S.plane + g] + bg[f]);
  }
  // pairwise tree over the block, carrying the compensation terms
  __shared__ double sh[8][256];
  for (int f = 0; f < 4; ++f) {
    sh[2 * f][threadIdx.x] = s[f];
    sh[2 * f + 1][threadIdx.x] = c[f];
  }
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w)
      for (int f = 0; f < 4; ++f) {
        double a = sh[2 * f][threadIdx.x], ca = sh[2 * f + 1][threadIdx.x];
        neumaier_add(a, ca, sh[2 * f][threadIdx.x + w]);
        sh[2 * f][threadIdx.x] = a;
        sh[2 * f + 1][threadIdx.x] = ca + sh[2 * f + 1][threadIdx.x + w];
      }
    __syncthreads();
  }
  if (threadIdx.x < 8) out[blockIdx.x * 8 + threadIdx.x] = sh[threadIdx.x][0];
}

// ---------------------------------------------------------------- arena
// Device memory for the state arena (arena.hpp).
struct DeviceMemory {
  static void *reserve(size_t n) {
    void *p = nullptr;
    if (cudaMalloc(&p, n) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    return p;
  }
  static void unreserve(void *p) { cudaFree(p); }
};

struct Pending {
  int64_t id;
  fv2d_request req;
  double submit_s;
};

struct Slot {
  bool used = false;
  int64_t id = -1;
  fv2d_request req;
  int bucket = 0, lane = 0, cfg = 0;
  int items = 0;  // work-list entries reserved for it (its items at the smallest band height)
  void *mem = nullptr;
  size_t bytes = 0;
  double submit_s = 0, admit_s = 0;
  double cons0[4] = {0, 0, 0, 0};
  double cells_done = 0;
  int steps_seen = 0;
};

struct Finished {
  fv2d_result res;
  std::vector<float> U;  // interior conservative offset planes, Ny x Nx each
  double gamma;
  double bg_r, bg_e;     // background of the offsets
};

}  // namespace

struct fv2d_server {
  fv2d_server_config cfg;
  int device = 0, num_sms = 0;
  cudaStream_t stream = nullptr;
  std::chrono::steady_clock::time_point t0;
  // simulation table
  int max_sims = 0;
  SimDev *d_sims = nullptr;
  SimDev *h_up = nullptr, *h_down = nullptr;  // pinned mirrors (uploads / readbacks)
  CUtensorMap *d_tmaps = nullptr, *h_tmaps = nullptr;
  std::vector<Slot> slots;
  std::vector<int> free_slots;
  // per-lane work lists (lane = bucket + kBuckets * family)
  WorkItem *d_work[kLanes] = {};
  int *d_nwork = nullptr, *h_nwork = nullptr;
  WorkItem *h_work[kLanes] = {};
  int work_cap[kLanes] = {};
  int items_in[kLanes] = {};  // work items of the resident requests, per lane
  // configuration per family and bucket (the extended family: one for every bucket)
  int fam_cfg[kFamilies][kBuckets] = {{1, 2, 3, 3}, {1, 2, 3, 3}, {-1, -1, -1, -1}};
  std::vector<int> cfg_grid;  // persistent grid per configuration (0: cannot run here)
  bool lists_dirty = true;
  int mask = 0;
  std::map<std::pair<int, int>, cudaGraphExec_t> graphs;  // (K, lane mask) -> graph
  double *d_cons = nullptr, *h_cons = nullptr;
  // kernel control words (BatchArgs::ctl): fault bits, tile-copy wait limit
  unsigned int *d_ctl = nullptr, *h_ctl = nullptr;
  std::atomic<uint32_t> wait_limit_req{0};  // test hook: a new wait limit for the worker to apply (0: none)
  float *h_stage = nullptr;
  size_t h_stage_size = 0;
  Arena<DeviceMemory> arena;
  // queues
  std::mutex mu;
  std::condition_variable cv;
  std::deque<Pending> queue;
  std::vector<fv2d_result> done_unpolled;
  std::unordered_map<int64_t, std::shared_ptr<const Finished>> finished;  // shared: get_prim reads outside mu
  int64_t next_id = 1;
  int64_t n_submitted = 0, n_admitted = 0, n_completed = 0, n_failed = 0;
  std::atomic<bool> stop{false};
  std::thread worker;
  double cell_updates = 0, busy_s = 0;  // written by the worker; published below under mu
  int replays = 0;
  int n_active = 0;  // resident requests (worker only)
  // copies for fv2d_server_get_stats, updated under mu
  struct Published {
    double cell_updates = 0, busy_s = 0, bytes_in_use = 0, bytes_reserved = 0;
    int replays = 0, active = 0;
    int64_t admitted = 0;
  } pub;
  double rate_est = 2e10;  // cell-updates/s, refined by measurement
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // the lanes' step chains run as parallel branches of a replay graph
  cudaStream_t bstream[kLanes] = {};
  cudaEvent_t ev_fork = nullptr, ev_join[kLanes] = {};
  double sched_cells = 0;  // cell-stages advanced per launch by the current work lists
  // failure state: `fault` is written by the worker alone; `broken`,
  // `fail_code` and `err` are set once, under mu, when the worker stops
  std::string fault;
  std::atomic<bool> inject{false};
  bool broken = false;
  int fail_code = FV2D_OK;
  std::string err;

  double now() const { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); }
};

namespace {

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void *ptr = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(ptr);
  }
  return fn;
}

const char *check_request(const fv2d_request &r) {
  const fv2d_params &p = r.params;
  if (r.struct_size != sizeof(fv2d_request)) return "fv2d_request.struct_size mismatch";
  if (const char *w = validate(p)) return w;
  if (p.Nx < kMinSide || p.Nx > kMaxSide || p.Ny < kMinSide || p.Ny > kMaxSide)
    return "Nx and Ny must be in [16, 8192]";
  if (!problem_valid(r.problem)) return "unknown problem";
  if (r.max_steps < 0) return "max_steps < 0";
  return nullptr;
}

// The extended family serves FSLP, the MUSCL-Hancock predictor, analytical
// gravity, B02 conductivity, the y-boundary conduction modes and the
// well-balanced y flux.
bool needs_ext(const fv2d_params &p) {
  return p.riemann_solver == FV2D_FSLP || p.reconstruction == FV2D_MUSCL_HANCOCK ||
         p.gravity_mode == FV2D_GRAV_ANALYTICAL || p.well_balanced_flux_at_y_bc ||
         (p.thermal_conductivity_active && (p.thermal_conductivity_mode != FV2D_TCM_CONSTANT ||
                                            p.bctc_ymin != FV2D_BCTC_NONE || p.bctc_ymax != FV2D_BCTC_NONE));
}
// The kernel family of a request: extended, else diffusive (constant
// conduction or viscosity), else plain.
int family_of(const fv2d_params &p) {
  if (needs_ext(p)) return FAM_EXT;
  return (p.thermal_conductivity_active || p.viscosity_active) ? FAM_DIFF : FAM_PLAIN;
}
bool needs_rows(const fv2d_params &p) {
  return p.gravity_mode == FV2D_GRAV_ANALYTICAL ||
         (p.thermal_conductivity_active && p.thermal_conductivity_mode != FV2D_TCM_CONSTANT);
}

// Background of the stored offsets: the median density and total energy of
// the initial condition, sampled on at most 64 x 64 cells (momenta have none:
// reflections negate them).
void background(const fv2d_request &r, float *bg_r, float *bg_e) {
  const fv2d_params &p = r.params;
  const int sx = std::max(1, p.Nx / 64), sy = std::max(1, p.Ny / 64);
  std::vector<double> rs, es;
  const Gas<double> g{p.gamma0, p.gamma0 - 1.0, 1.0 / (p.gamma0 - 1.0), 0.0};
  for (int j = sy / 2; j < p.Ny; j += sy)
    for (int i = sx / 2; i < p.Nx; i += sx) {
      double q[4];
      init_cell(p, r.problem, i, j, q);
      const S4<double> u = prim_to_cons(S4<double>{q[0], q[1], q[2], q[3]}, g);
      rs.push_back(u.r);
      es.push_back(u.p);
    }
  auto median = [](std::vector<double> &v) {
    std::nth_element(v.begin(), v.begin() + v.size() / 2, v.end());
    return v[v.size() / 2];
  };
  const double mr = median(rs), me = median(es);
  *bg_r = std::isfinite(mr) ? (float)mr : 0.f;
  *bg_e = std::isfinite(me) ? (float)me : 0.f;
}

// Synchronises the worker's stream.  A failure is recorded in s->fault: the
// context is then unusable, and the worker stops after this iteration.
bool sync_stream(fv2d_server *s) {
  const cudaError_t e = cudaStreamSynchronize(s->stream);
  if (e == cudaSuccess) return true;
  if (s->fault.empty()) s->fault = std::string("CUDA: ") + cudaGetErrorString(e);
  return false;
}

// Device bytes of a simulation: two buffers of four planes with the ghost
// ring, then (when the request needs it) its per-row table.
size_t state_bytes(const fv2d_params &p, int *pitch, long long *plane, size_t *rows_off) {
  *pitch = (p.Nx + 4 + 31) / 32 * 32;
  *plane = (long long)(p.Ny + 4) * *pitch;
  const size_t planes = sizeof(float) * 8 * (size_t)*plane;  // two buffers x four planes
  *rows_off = (planes + 255) & ~size_t(255);
  return needs_rows(p) ? *rows_off + sizeof(float) * kRowStride * (size_t)p.Ny : planes;
}

int lane_cfg(const fv2d_server *s, int lane) { return s->fam_cfg[lane / kBuckets][lane % kBuckets]; }

// Lane of a request: its grid-size bucket + kBuckets * its family; with
// single_launch every request of a family shares the family's first lane
// (one work list, one launch per step).
int lane_of(const fv2d_server_config &cfg, int bucket, int family) {
  return (cfg.single_launch ? 0 : bucket) + family * kBuckets;
}

// Grow lane b's work-list buffers to hold `need` items.  New buffers are
// allocated before the old ones are released, so a failure leaves the lists
// as they were.
bool reserve_work(fv2d_server *s, int b, int need) {
  if (need <= s->work_cap[b]) return true;
  int cap = std::max(1024, s->work_cap[b]);
  while (cap < need) cap *= 2;
  WorkItem *d = nullptr, *h = nullptr;
  if (cudaMalloc(&d, sizeof(WorkItem) * cap) != cudaSuccess ||
      cudaMallocHost(&h, sizeof(WorkItem) * cap) != cudaSuccess) {
    cudaGetLastError();
    if (d) cudaFree(d);
    return false;
  }
  cudaStreamSynchronize(s->stream);  // the next rebuild fills the new lists
  if (s->d_work[b]) cudaFree(s->d_work[b]);
  if (s->h_work[b]) cudaFreeHost(s->h_work[b]);
  s->d_work[b] = d;
  s->h_work[b] = h;
  s->work_cap[b] = cap;
  for (auto &g : s->graphs) cudaGraphExecDestroy(g.second);  // kernel arguments changed
  s->graphs.clear();
  s->lists_dirty = true;
  return true;
}

// Admit one request into a free slot; returns the slot, or -1 when it does
// not fit (HBM budget, table or work-list capacity).
int admit(fv2d_server *s, const Pending &pd) {
  const NvtxRange nvtx_range("fv2d_server admit");
  if (s->free_slots.empty()) return -1;
  const fv2d_request &r = pd.req;
  const fv2d_params &p = r.params;
  const int Nx = p.Nx, Ny = p.Ny;
  int pitch;
  long long plane;
  size_t rows_off;
  const size_t bytes = state_bytes(p, &pitch, &plane, &rows_off);
  const int bucket = bucket_of(Nx, Ny);
  const int family = family_of(p);
  const bool ext = family == FAM_EXT;
  const int lane = lane_of(s->cfg, bucket, family);
  const int cfg = lane_cfg(s, lane);
  int tx, ty, nt, staging;
  batch_cfg_info(cfg, &tx, &ty, &nt, &staging, nullptr, nullptr, nullptr);
  // the march kernels' band height changes with the lane's contents: room for
  // the most items it can take
  const int items = ((Nx + tx - 1) / tx) * ((Ny + (staging == 2 ? kMinBand : ty) - 1) / (staging == 2 ? kMinBand : ty));
  float bg_r = 0.f, bg_e = 0.f;
  if (pd.id > 0) background(r, &bg_r, &bg_e);  // the autotuner's synthetic states need none
  // state memory first: a request that does not fit must not grow the work
  // lists (that synchronises the stream and drops the captured graphs)
  void *mem = s->arena.alloc(bytes);
  if (!mem) return -1;
  if (!reserve_work(s, lane, s->items_in[lane] + items)) {
    s->arena.release(mem, bytes);
    return -1;
  }
  s->items_in[lane] += items;
  const int slot = s->free_slots.back();
  s->free_slots.pop_back();
  Slot &sl = s->slots[slot];
  sl.used = true;
  sl.id = pd.id;
  sl.req = r;
  sl.bucket = bucket;
  sl.lane = lane;
  sl.cfg = cfg;
  sl.items = items;
  sl.mem = mem;
  sl.bytes = bytes;
  sl.submit_s = pd.submit_s;
  sl.admit_s = s->now();
  sl.cells_done = 0;
  sl.steps_seen = 0;

  SimDev &d = s->h_up[slot];
  std::memset(&d, 0, sizeof(d));
  d.U[0] = static_cast<float *>(mem);
  d.U[1] = static_cast<float *>(mem) + 4 * plane;
  d.rows = needs_rows(p) ? reinterpret_cast<const float *>(static_cast<char *>(mem) + rows_off) : nullptr;
  d.plane = plane;
  d.pitch = pitch;
  d.Nx = Nx;
  d.Ny = Ny;
  d.ntx = (Nx + tx - 1) / tx;
  d.band = ty;  // the march lanes' band is set by rebuild_lists
  d.nty = (Ny + ty - 1) / ty;
  d.cur = 0;
  d.status = SIM_ACTIVE;
  d.step = 0;
  d.max_steps = r.max_steps;
  d.ts = p.time_stepping == FV2D_TS_RK2 ? 1 : 0;
  d.stage = 0;
  d.t = 0.0;
  d.dt = 0.0;
  d.tend = r.tend > 0 ? r.tend : INFINITY;
  d.eps = p.epsilon;
  parabolic_inv_dt(p, &d.inv_tc, &d.inv_visc);
  d.cfl = p.CFL;
  d.gamma = (float)p.gamma0;
  d.gm1 = (float)(p.gamma0 - 1.0);
  d.entho = (float)(1.0 / (p.gamma0 - 1.0));
  d.fslp_K = (float)p.fslp_K;
  const double dx = (p.xmax - p.xmin) / Nx, dy = (p.ymax - p.ymin) / Ny;
  d.dx = (float)dx;
  d.dy = (float)dy;
  d.inv_dx = (float)(1.0 / dx);
  d.inv_dy = (float)(1.0 / dy);
  d.gx = (float)p.gx;
  d.gy = (float)p.gy;
  d.gdx = (float)(p.gx * dx);
  d.gdy = (float)(p.gy * dy);
  d.kappa = (float)p.kappa;
  d.mu = (float)p.mu;
  d.bg_r = bg_r;
  d.bg_e = bg_e;
  d.rs = p.riemann_solver == FV2D_HLL ? RS_HLL : (p.riemann_solver == FV2D_FSLP ? RS_FSLP : RS_HLLC);
  d.recon = p.reconstruction == FV2D_PLM ? BR_PLM : (p.reconstruction == FV2D_MUSCL_HANCOCK ? BR_MH : BR_PCM);
  d.ext = ext ? 1 : 0;
  d.bcx = p.boundary_x;
  d.bcy = p.boundary_y;
  d.grav = p.gravity_mode == FV2D_GRAV_CONSTANT ? BG_CONST : (p.gravity_mode == FV2D_GRAV_ANALYTICAL ? BG_ROW : BG_NONE);
  d.tc = !p.thermal_conductivity_active ? BK_NONE
                                        : (p.thermal_conductivity_mode == FV2D_TCM_CONSTANT ? BK_CONST : BK_ROW);
  d.visc = p.viscosity_active ? 1 : 0;
  d.wb = p.well_balanced_flux_at_y_bc ? 1 : 0;
  d.bctc_lo = p.thermal_conductivity_active ? p.bctc_ymin : FV2D_BCTC_NONE;
  d.bctc_hi = p.thermal_conductivity_active ? p.bctc_ymax : FV2D_BCTC_NONE;
  d.bctc_lo_v = (float)p.bctc_ymin_value;
  d.bctc_hi_v = (float)p.bctc_ymax_value;
  d.lowmach = r.lowmach ? 1 : 0;
  d.tma_ok = 0;
  if (staging == 1) {  // TMA staging needs the tensor maps
    PFN_cuTensorMapEncodeTiled_v12000 enc = encode_fn();
    bool ok = enc != nullptr;
    for (int b = 0; b < 2 && ok; ++b) {
      cuuint64_t dims[3] = {(cuuint64_t)(Nx + 4), (cuuint64_t)(Ny + 4), 4};
      cuuint64_t strides[2] = {(cuuint64_t)pitch * 4, (cuuint64_t)plane * 4};
      cuuint32_t box[3] = {(cuuint32_t)(tx + 4), (cuuint32_t)(ty + 4), 4};
      cuuint32_t es[3] = {1, 1, 1};
      ok = enc(&s->h_tmaps[2 * slot + b], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, d.U[b], dims, strides, box, es,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
    }
    d.tma_ok = ok ? 1 : 0;
    if (ok)
      cudaMemcpyAsync(&s->d_tmaps[2 * slot], &s->h_tmaps[2 * slot], 2 * sizeof(CUtensorMap), cudaMemcpyHostToDevice,
                      s->stream);
  }
  cudaMemcpyAsync(&s->d_sims[slot], &d, sizeof(SimDev), cudaMemcpyHostToDevice, s->stream);
  const long long cells_padded = (long long)(Nx + 4) * (Ny + 4);
  ic_kernel<<<(unsigned)((cells_padded + 255) / 256), 256, 0, s->stream>>>(p, r.problem, d.U[0], plane, pitch, Nx,
                                                                              Ny, bg_r, bg_e);
  if (d.rows)
    rows_kernel<<<(Ny + 127) / 128, 128, 0, s->stream>>>(p, const_cast<float *>(d.rows));
  const int nb = (int)std::min<long long>(1024, ((long long)Nx * Ny + 255) / 256);
  first_dt_kernel<<<nb, 256, 0, s->stream>>>(s->d_sims, slot);
  first_dt_finish<<<1, 1, 0, s->stream>>>(s->d_sims, slot);
  if (pd.id > 0)  // the autotuner's synthetic states need no sums
    cons_kernel<<<kConsBlocks, 256, 0, s->stream>>>(s->d_sims, slot, s->d_cons + (size_t)slot * kConsBlocks * 8);
  s->n_admitted++;
  s->n_active++;
  s->lists_dirty = true;
  return slot;
}

void sum_cons(const double *part, double out[4]) {
  for (int f = 0; f < 4; ++f) {
    double ss = 0, cc = 0;
    for (int b = 0; b < kConsBlocks; ++b) {
      const double x = part[(b * 4 + f) * 2];
      const double t = ss + x;
      cc += (std::fabs(ss) >= std::fabs(x)) ? (ss - t) + x : (x - t) + ss;
      ss = t;
      cc += part[(b * 4 + f) * 2 + 1];
    }
    out[f] = ss + cc;
  }
}

// Initial conservation sums of the slots admitted since the last replay.
void read_initial_cons(fv2d_server *s, const std::vector<int> &fresh) {
  if (fresh.empty()) return;
  for (int slot : fresh)
    cudaMemcpyAsync(s->h_cons + (size_t)slot * kConsBlocks * 8, s->d_cons + (size_t)slot * kConsBlocks * 8,
                    sizeof(double) * kConsBlocks * 8, cudaMemcpyDeviceToHost, s->stream);
  if (!sync_stream(s)) return;
  for (int slot : fresh) {
    Slot &sl = s->slots[slot];
    const fv2d_params &p = sl.req.params;
    const double area = ((p.xmax - p.xmin) / p.Nx) * ((p.ymax - p.ymin) / p.Ny);
    sum_cons(s->h_cons + (size_t)slot * kConsBlocks * 8, sl.cons0);
    for (int f = 0; f < 4; ++f) sl.cons0[f] *= area;
  }
}

// Copy the worker's counters for fv2d_server_get_stats; the caller holds mu.
void publish_locked(fv2d_server *s) {
  s->pub.cell_updates = s->cell_updates;
  s->pub.busy_s = s->busy_s;
  s->pub.replays = s->replays;
  s->pub.admitted = s->n_admitted;
  s->pub.active = s->n_active;
  s->pub.bytes_in_use = (double)s->arena.in_use;
  s->pub.bytes_reserved = (double)s->arena.reserved;
}

// Launches a step of this request takes (SSP-RK2: two stages).
int stages_of(const fv2d_params &p) { return p.time_stepping == FV2D_TS_RK2 ? 2 : 1; }

// Remaining cell-updates of a resident request: its remaining steps (the
// step limit, or the time limit at the last dt when that comes first) times
// its cells and stages.
double remaining_work(const fv2d_server *s, int slot) {
  const Slot &sl = s->slots[slot];
  const double cells = (double)sl.req.params.Nx * sl.req.params.Ny * stages_of(sl.req.params);
  double steps = (double)sl.req.max_steps - sl.steps_seen;
  if (sl.steps_seen > 0 && sl.req.tend > 0) {
    const SimDev &d = s->h_down[slot];
    if (d.dt > 0) steps = std::min(steps, std::ceil((sl.req.tend - d.t) / d.dt));
  }
  return std::max(steps, 1.0) * cells;
}

// Band height of a march lane for the simulations it is about to run
// (schedule.hpp); the tile kernels keep their tile height.  A simulation's
// results do not depend on the band: every face is computed by the same code
// whichever band holds it.
int lane_band(const fv2d_server *s, int lane, const std::vector<int> &slots) {
  const int c = lane_cfg(s, lane);
  int tx, ty, nt, staging;
  batch_cfg_info(c, &tx, &ty, &nt, &staging, nullptr, nullptr, nullptr);
  if (staging != 2 || slots.empty()) return ty;
  if (s->cfg.band_rows > 0) return s->cfg.band_rows;
  std::vector<BandGrid> grids;
  grids.reserve(slots.size());
  for (int k : slots) grids.push_back(BandGrid{s->h_up[k].ntx, s->h_up[k].Ny});
  return choose_band(grids, (double)s->cfg_grid[c] * (nt / 32));
}

void rebuild_lists(fv2d_server *s) {
  std::vector<WorkItem> lists[kLanes];
  // shortest remaining work first, up to about active_cells cells per step
  // (every resident request when active_cells is 0)
  std::vector<Candidate> cand;
  for (int k = 0; k < s->max_sims; ++k)
    if (s->slots[k].used) {
      const fv2d_params &p = s->slots[k].req.params;
      cand.push_back({k, s->cfg.active_cells > 0 ? remaining_work(s, k) : 0.0,
                      (double)p.Nx * p.Ny * stages_of(p)});
    }
  const std::vector<int> run = select_active(std::move(cand), s->cfg.active_cells);
  // interleave work items of the simulations of a lane so that a CTA's
  // consecutive items belong to different simulations
  std::vector<int> per_lane[kLanes];
  s->sched_cells = 0;
  for (int k : run) {
    per_lane[s->slots[k].lane].push_back(k);
    s->sched_cells += (double)s->slots[k].req.params.Nx * s->slots[k].req.params.Ny;
  }
  s->mask = 0;
  for (int b = 0; b < kLanes; ++b) {
    const int band = lane_band(s, b, per_lane[b]);
    for (int slot : per_lane[b]) {
      SimDev &u = s->h_up[slot];
      if (u.band != band) {  // nty and band, adjacent in the table entry
        u.band = band;
        u.nty = (u.Ny + band - 1) / band;
        cudaMemcpyAsync(&s->d_sims[slot].nty, &u.nty, 2 * sizeof(int), cudaMemcpyHostToDevice, s->stream);
      }
    }
    for (int slot : per_lane[b]) {
      const SimDev &d = s->h_up[slot];
      for (int ty = 0; ty < d.nty; ++ty)
        for (int tx = 0; tx < d.ntx; ++tx) lists[b].push_back(WorkItem{slot, (short)tx, (short)ty});
    }
    if (!lists[b].empty()) s->mask |= 1 << b;
    // admission reserved room for every resident request's items
    const int n = std::min((int)lists[b].size(), s->work_cap[b]);
    s->h_nwork[b] = n;
    if (n) {
      std::memcpy(s->h_work[b], lists[b].data(), sizeof(WorkItem) * n);
      cudaMemcpyAsync(s->d_work[b], s->h_work[b], sizeof(WorkItem) * n, cudaMemcpyHostToDevice, s->stream);
    }
  }
  cudaMemcpyAsync(s->d_nwork, s->h_nwork, sizeof(int) * kLanes, cudaMemcpyHostToDevice, s->stream);
  s->lists_dirty = false;
}

cudaError_t launch_step(fv2d_server *s, int mask) {
  for (int b = 0; b < kLanes; ++b) {
    if (!(mask & (1 << b))) continue;
    BatchArgs a{s->d_sims, s->d_work[b], s->d_nwork + b, s->d_tmaps, s->d_ctl};
    const int c = lane_cfg(s, b);
    cudaError_t e = batch_launch(c, s->cfg_grid[c], s->stream, a);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaGraphExec_t get_graph(fv2d_server *s, int K, int mask) {
  auto key = std::make_pair(K, mask);
  auto it = s->graphs.find(key);
  if (it != s->graphs.end()) return it->second;
  cudaGraph_t g;
  if (cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return nullptr;
  // one branch per lane: a request's steps depend only on its own previous
  // step, so the lanes' chains are independent and a small bucket's
  // kernels can fill the SMs that a large one's leave idle
  cudaEventRecord(s->ev_fork, s->stream);
  for (int b = 0; b < kLanes; ++b) {
    if (!(mask & (1 << b))) continue;
    cudaStreamWaitEvent(s->bstream[b], s->ev_fork, 0);
    BatchArgs a{s->d_sims, s->d_work[b], s->d_nwork + b, s->d_tmaps, s->d_ctl};
    const int c = lane_cfg(s, b);
    for (int k = 0; k < K; ++k) batch_launch(c, s->cfg_grid[c], s->bstream[b], a);
    cudaEventRecord(s->ev_join[b], s->bstream[b]);
    cudaStreamWaitEvent(s->stream, s->ev_join[b], 0);
  }
  if (cudaStreamEndCapture(s->stream, &g) != cudaSuccess) return nullptr;
  cudaGraphExec_t ex = nullptr;
  if (cudaGraphInstantiate(&ex, g, 0) != cudaSuccess) ex = nullptr;
  cudaGraphDestroy(g);
  if (ex) s->graphs[key] = ex;
  return ex;
}

// Retire the finished simulations of one replay: final conservation sums and
// state copies are queued for all of them, then one synchronisation.
void retire_all(fv2d_server *s, const std::vector<int> &done) {
  if (done.empty()) return;
  const NvtxRange nvtx_range("fv2d_server retire");
  size_t need = 0;
  std::vector<size_t> off(done.size());
  for (size_t k = 0; k < done.size(); ++k) {
    off[k] = need;
    need += 4 * (size_t)s->h_down[done[k]].Nx * s->h_down[done[k]].Ny;
  }
  if (s->h_stage_size < need * sizeof(float)) {
    if (s->h_stage) cudaFreeHost(s->h_stage);
    s->h_stage = nullptr;
    s->h_stage_size = 0;
    if (cudaMallocHost(&s->h_stage, need * sizeof(float)) == cudaSuccess)
      s->h_stage_size = need * sizeof(float);
    else
      cudaGetLastError();
  }
  // page-locked staging when it could be had, else pageable memory (the same
  // copies, without overlap); with neither, the requests complete with
  // FV2D_ERR_NOMEM and no final state
  std::vector<float> pageable;
  float *stage = s->h_stage;
  if (!stage) {
    try {
      pageable.resize(need);
      stage = pageable.data();
    } catch (const std::bad_alloc &) {
    }
  }
  for (size_t k = 0; k < done.size(); ++k) {
    const int slot = done[k];
    const SimDev &d = s->h_down[slot];
    const int Nx = d.Nx, Ny = d.Ny;
    cons_kernel<<<kConsBlocks, 256, 0, s->stream>>>(s->d_sims, slot, s->d_cons + (size_t)slot * kConsBlocks * 8);
    cudaMemcpyAsync(s->h_cons + (size_t)slot * kConsBlocks * 8, s->d_cons + (size_t)slot * kConsBlocks * 8,
                    sizeof(double) * kConsBlocks * 8, cudaMemcpyDeviceToHost, s->stream);
    for (int f = 0; f < 4 && stage; ++f)
      cudaMemcpy2DAsync(stage + off[k] + (size_t)f * Nx * Ny, sizeof(float) * Nx,
                        d.U[d.cur] + f * d.plane + 2 * d.pitch + 2, sizeof(float) * d.pitch, sizeof(float) * Nx, Ny,
                        cudaMemcpyDeviceToHost, s->stream);
    // mark the device slot free so stale work-list entries are skipped
    s->h_up[slot].status = SIM_FREE;
    cudaMemcpyAsync(&s->d_sims[slot].status, &s->h_up[slot].status, sizeof(int), cudaMemcpyHostToDevice,
                    s->stream);
  }
  if (!sync_stream(s)) return;  // the slots stay resident; the worker fails them
  const double t_done = s->now();
  for (size_t k = 0; k < done.size(); ++k) {
    const int slot = done[k];
    const SimDev &d = s->h_down[slot];
    Slot &sl = s->slots[slot];
    const size_t cells = (size_t)d.Nx * d.Ny;
    Finished fin;
    fv2d_result &r = fin.res;
    std::memset(&r, 0, sizeof(r));
    r.id = sl.id;
    r.status = d.status == SIM_DONE ? FV2D_OK : (d.dev_err ? FV2D_ERR_CUDA : FV2D_ERR_NUMERIC);
    r.steps = d.step;
    r.t = d.t;
    r.submit_s = sl.submit_s;
    r.admit_s = sl.admit_s;
    r.negatives = d.negatives;
    r.Nx = d.Nx;
    r.Ny = d.Ny;
    r.bucket = sl.bucket;
    r.lane = sl.lane;
    const fv2d_params &p = sl.req.params;
    const double area = ((p.xmax - p.xmin) / p.Nx) * ((p.ymax - p.ymin) / p.Ny);
    double c1[4];
    sum_cons(s->h_cons + (size_t)slot * kConsBlocks * 8, c1);
    for (int f = 0; f < 4; ++f) {
      r.cons0[f] = sl.cons0[f];
      r.cons1[f] = c1[f] * area;
    }
    bool kept = false;
    if (stage) {
      try {
        fin.U.assign(stage + off[k], stage + off[k] + 4 * cells);
        kept = true;
      } catch (const std::bad_alloc &) {
      }
    }
    if (!kept && r.status == FV2D_OK) r.status = FV2D_ERR_NOMEM;
    fin.gamma = p.gamma0;
    fin.bg_r = d.bg_r;
    fin.bg_e = d.bg_e;
    r.done_s = t_done;
    s->arena.release(sl.mem, sl.bytes);
    s->items_in[sl.lane] -= sl.items;
    s->n_active--;
    sl.used = false;
    sl.mem = nullptr;
    s->free_slots.push_back(slot);
    s->lists_dirty = true;
    std::lock_guard<std::mutex> lock(s->mu);
    publish_locked(s);  // before the completion count that fv2d_server_drain waits for
    if (r.status == FV2D_OK)
      s->n_completed++;
    else
      s->n_failed++;
    try {
      s->done_unpolled.push_back(r);
      if (kept) s->finished.emplace(r.id, std::make_shared<const Finished>(std::move(fin)));
    } catch (const std::bad_alloc &) {  // counted; its record or final state is lost
    }
  }
  s->cv.notify_all();
}

// Replay K steps of every active simulation and retire the finished ones.
// Returns false when nothing was active.
bool run_once(fv2d_server *s, int K_fixed) {
  const NvtxRange nvtx_range("fv2d_server replay");
  bool any = false;
  for (int k = 0; k < s->max_sims; ++k)
    if (s->slots[k].used) {
      any = true;
      break;
    }
  if (!any) return false;
  if (s->lists_dirty) rebuild_lists(s);
  int K = K_fixed;
  if (K <= 0) {
    const double step_s = s->sched_cells / s->rate_est;
    K = 1;
    while (K < 64 && (K * 2) * step_s < 3e-3) K *= 2;
  }
  cudaGraphExec_t g = get_graph(s, K, s->mask);
  const double t_start = s->now();
  cudaEventRecord(s->ev0, s->stream);
  if (g)
    cudaGraphLaunch(g, s->stream);
  else
    for (int k = 0; k < K; ++k) launch_step(s, s->mask);
  cudaEventRecord(s->ev1, s->stream);
  int hi = 0;
  for (int k = 0; k < s->max_sims; ++k)
    if (s->slots[k].used) hi = k + 1;
  cudaMemcpyAsync(s->h_down, s->d_sims, sizeof(SimDev) * hi, cudaMemcpyDeviceToHost, s->stream);
  cudaMemcpyAsync(s->h_ctl, s->d_ctl, sizeof(unsigned int), cudaMemcpyDeviceToHost, s->stream);
  if (!sync_stream(s)) return true;
  if (s->h_ctl[0]) {  // a CTA stopped with a tile copy in flight: shared memory can no longer be trusted
    s->fault = "device: a tile copy of the served step did not complete within its bounded waits";
    return true;
  }
  float ms = 0;
  cudaEventElapsedTime(&ms, s->ev0, s->ev1);
  s->replays++;
  s->busy_s += s->now() - t_start;
  double cells = 0;
  std::vector<int> done;
  for (int k = 0; k < hi; ++k) {
    Slot &sl = s->slots[k];
    if (!sl.used) continue;
    const SimDev &d = s->h_down[k];
    const int new_steps = d.step - sl.steps_seen;
    cells += (double)d.Nx * d.Ny * new_steps;
    sl.steps_seen = d.step;
    if (d.status == SIM_DONE || d.status == SIM_FAILED) done.push_back(k);
  }
  s->cell_updates += cells;
  if (ms > 0.05 && cells > 0) s->rate_est = 0.5 * s->rate_est + 0.5 * (cells / (ms * 1e-3));
  retire_all(s, done);
  std::lock_guard<std::mutex> lock(s->mu);
  publish_locked(s);
  return true;
}

// The worker cannot go on: its stream failed (the CUDA context is then
// unusable), or host memory ran out while it changed its tables.  Every
// resident request, every queued one and the ones in `extra` (taken from the
// queue and not yet admitted) complete with `code`; later submissions are
// refused.  Device memory stays with the server until fv2d_server_destroy.
void fail_all(fv2d_server *s, int code, const std::vector<Pending> &extra) noexcept {
  const double t = s->now();
  std::lock_guard<std::mutex> lock(s->mu);
  s->broken = true;
  s->fail_code = code;
  try {
    s->err = s->fault.empty() ? std::string("service stopped") : s->fault;
  } catch (const std::bad_alloc &) {
  }
  auto post = [&](int64_t id, double submit_s, double admit_s, const fv2d_params &p, int steps) {
    fv2d_result r;
    std::memset(&r, 0, sizeof(r));
    r.id = id;
    r.status = code;
    r.steps = steps;
    r.submit_s = submit_s;
    r.admit_s = admit_s;
    r.done_s = t;
    r.Nx = p.Nx;
    r.Ny = p.Ny;
    r.bucket = bucket_of(p.Nx, p.Ny);
    r.lane = lane_of(s->cfg, r.bucket, family_of(p));
    s->n_failed++;
    try {
      s->done_unpolled.push_back(r);
    } catch (const std::bad_alloc &) {  // counted; its record is lost
    }
  };
  for (Slot &sl : s->slots)
    if (sl.used) {
      post(sl.id, sl.submit_s, sl.admit_s, sl.req.params, sl.steps_seen);
      sl.used = false;
    }
  for (const Pending &pd : s->queue) post(pd.id, pd.submit_s, -1.0, pd.req.params, 0);
  for (const Pending &pd : extra) post(pd.id, pd.submit_s, -1.0, pd.req.params, 0);
  s->queue.clear();
  s->n_active = 0;
  publish_locked(s);
  s->cv.notify_all();
}

void worker_main(fv2d_server *s) {
  cudaSetDevice(s->device);
  while (!s->stop.load()) {
    std::vector<Pending> take, keep;
    size_t next = 0;  // entries of `take` before this one were admitted or moved to `keep`
    try {
      {
        std::unique_lock<std::mutex> lock(s->mu);
        bool active = false;
        for (auto &sl : s->slots)
          if (sl.used) {
            active = true;
            break;
          }
        if (!active && s->queue.empty())
          s->cv.wait_for(lock, std::chrono::milliseconds(20));
        take.assign(s->queue.begin(), s->queue.end());
        s->queue.clear();
      }
      // admission: first in, first out; a request that does not fit waits and
      // smaller ones behind it may pass
      std::vector<int> fresh;
      fresh.reserve(take.size());  // no allocation once a request is admitted
      keep.reserve(take.size());
      for (; next < take.size(); ++next) {
        const int slot = admit(s, take[next]);
        if (slot >= 0)
          fresh.push_back(slot);
        else
          keep.push_back(take[next]);
      }
      if (!keep.empty()) {
        std::lock_guard<std::mutex> lock(s->mu);
        std::deque<Pending> q(keep.begin(), keep.end());
        q.insert(q.end(), s->queue.begin(), s->queue.end());
        s->queue.swap(q);
      }
      keep.clear();
      take.clear();
      next = 0;
      read_initial_cons(s, fresh);
      if (!fresh.empty()) {
        std::lock_guard<std::mutex> lock(s->mu);
        publish_locked(s);
      }
      if (const uint32_t lim = s->wait_limit_req.exchange(0)) {  // test hook (fv2d_server_set_tile_wait_limit)
        s->h_ctl[1] = lim == UINT32_MAX ? 0u : lim;
        cudaMemcpyAsync(s->d_ctl + 1, s->h_ctl + 1, sizeof(unsigned int), cudaMemcpyHostToDevice, s->stream);
      }
      if (s->fault.empty()) run_once(s, s->cfg.steps_per_replay);
      if (s->fault.empty() && s->inject.exchange(false)) s->fault = "simulated failure (fv2d_server_inject_fault)";
      if (!s->fault.empty()) {
        fail_all(s, FV2D_ERR_CUDA, {});
        return;
      }
    } catch (const std::exception &e) {
      std::vector<Pending> extra;
      try {
        extra = keep;
        extra.insert(extra.end(), take.begin() + next, take.end());
        s->fault = std::string("host: ") + e.what();
      } catch (const std::bad_alloc &) {
      }
      fail_all(s, FV2D_ERR_NOMEM, extra);
      return;
    }
  }
}

// One autotuner trial: nsims synthetic Sedov requests of Nx x Ny (PLM +
// HLLC; with constant conduction and viscosity for the diffusive family)
// stepped with the bucket's current configuration; returns the rate in
// cell-updates/s, or -1 when the trial could not run.  Leaves the server
// empty.
double autotune_trial(fv2d_server *s, int family, int Nx, int Ny, int nsims) {
  for (int k = 0; k < nsims; ++k) {
    Pending pd;
    pd.id = -1 - k;
    std::memset(&pd.req, 0, sizeof(pd.req));
    pd.req.struct_size = sizeof(fv2d_request);
    pd.req.problem = FV2D_PB_SEDOV;
    params_default(&pd.req.params);
    pd.req.params.Nx = Nx;
    pd.req.params.Ny = Ny;
    pd.req.params.gamma0 = 1.4;
    pd.req.params.reconstruction = FV2D_PLM;
    pd.req.params.riemann_solver = FV2D_HLLC;
    if (family == FAM_DIFF) {
      pd.req.params.thermal_conductivity_active = 1;
      pd.req.params.kappa = 1e-4;
      pd.req.params.viscosity_active = 1;
      pd.req.params.mu = 1e-4;
    }
    pd.req.max_steps = 1 << 30;
    pd.req.tend = 0;
    pd.submit_s = 0;
    if (admit(s, pd) < 0) break;
  }
  rebuild_lists(s);
  for (int k = 0; k < 2; ++k) launch_step(s, s->mask);
  cudaEventRecord(s->ev0, s->stream);
  const int steps = 12;
  for (int k = 0; k < steps; ++k) launch_step(s, s->mask);
  cudaEventRecord(s->ev1, s->stream);
  cudaStreamSynchronize(s->stream);
  float ms = 0;
  cudaEventElapsedTime(&ms, s->ev0, s->ev1);
  double cells = 0;
  for (int k = 0; k < s->max_sims; ++k)
    if (s->slots[k].used) cells += (double)Nx * Ny;
  const bool ok = cudaGetLastError() == cudaSuccess && cells > 0 && ms > 0;
  for (int k = 0; k < s->max_sims; ++k)
    if (s->slots[k].used) {
      s->arena.release(s->slots[k].mem, s->slots[k].bytes);
      s->slots[k].used = false;
      s->h_up[k].status = SIM_FREE;
      s->free_slots.push_back(k);
    }
  cudaMemcpyAsync(s->d_sims, s->h_up, sizeof(SimDev) * s->max_sims, cudaMemcpyHostToDevice, s->stream);
  s->n_admitted = 0;
  s->n_active = 0;
  for (int q = 0; q < kLanes; ++q) s->items_in[q] = 0;
  s->lists_dirty = true;
  return ok ? cells * steps / (ms * 1e-3) : -1.0;
}

// Per family (plain, diffusive), the configuration that runs a mixture of
// requests in the least time, used for every bucket of the family.  The
// mixture holds one request per bucket (sides 96, 192, 384, 768: as many
// requests of each size, like sides spread log-uniformly, so that the cells
// and the time are mostly the large grids'); each bucket's rate is measured
// on a batch of about 24e6 cells of its size, and the largest bucket's as the
// geometric mean of that batch and one grid of 1024 x 3072 (the batch alone
// when the HBM budget cannot hold the grid), since it also holds single grids
// of millions of cells, which favour other work-item shapes.  One
// configuration per family: lanes that ran different kernels side by side
// (parallel graph branches) measured slower on the request stream than either
// kernel alone, and per-bucket choices from short trials changed from one
// start to the next.  The trials run under the service's own scheduling cap
// (active_cells), so a configuration is measured at the load its lanes will
// carry: on the 512-request stream at 8e6 cells per step the one-column march
// (smaller work items, more resident warps) gave p50 0.089 s against 0.103 s
// for the two-column one, which wins on full lanes (the same stream submitted
// at once: 50.1 against 48.9 G cell-updates/s).
void autotune(fv2d_server *s) {
  const int rep[kBuckets] = {96, 192, 384, 768};
  const int ncfg = num_cfgs();
  for (int f : {FAM_PLAIN, FAM_DIFF}) {
    double best = -1;
    int best_cfg = s->fam_cfg[f][kBuckets - 1];
    for (int c = 0; c < ncfg; ++c) {
      if (!s->cfg_grid[c] || !((cfg_fams(c) >> f) & 1)) continue;  // the family's configurations
      for (int b = 0; b < kBuckets; ++b) s->fam_cfg[f][b] = c;
      double cells = 0, time = 0;  // one request of each bucket
      bool ok = true;
      for (int b = 0; b < kBuckets && ok; ++b) {
        const int N = rep[b];
        const int nsims = std::max(2, std::min(256, (int)(24e6 / ((double)N * N))));
        double r = autotune_trial(s, f, N, N, nsims);
        if (b == kBuckets - 1 && r > 0) {
          const double single = autotune_trial(s, f, 1024, 3072, 1);  // -1 when the budget cannot hold it
          if (single > 0) r = std::sqrt(r * single);
        }
        ok = r > 0;
        cells += (double)N * N;
        time += ok ? (double)N * N / r : 0.0;
      }
      if (!ok) continue;
      const double score = cells / time;
      if (score > best) {
        best = score;
        best_cfg = c;
      }
    }
    for (int b = 0; b < kBuckets; ++b) s->fam_cfg[f][b] = best_cfg;
  }
  cudaStreamSynchronize(s->stream);
  s->free_slots.clear();
  for (int k = s->max_sims - 1; k >= 0; --k) s->free_slots.push_back(k);
}

}  // namespace

extern "C" {

const char *fv2d_server_config_name(int index) {
  if (index < 0 || index >= batch_num_cfgs()) return nullptr;
  const char *name;
  batch_cfg_info(index, nullptr, nullptr, nullptr, nullptr, nullptr, &name, nullptr);
  return name;
}

int fv2d_server_config_families(int index) {
  if (index < 0 || index >= batch_num_cfgs()) return -1;
  return cfg_fams(index);
}

int fv2d_server_create(const fv2d_server_config *cfg, fv2d_server **out) {
  if (!cfg || !out || cfg->struct_size != sizeof(fv2d_server_config)) return FV2D_ERR_INVALID;
  if (cfg->max_sims <= 0 || cfg->max_sims > 16384 || !(cfg->budget_bytes > 0)) return FV2D_ERR_INVALID;
  if (!(cfg->active_cells >= 0) || std::isinf(cfg->active_cells)) return FV2D_ERR_INVALID;
  if (cfg->single_launch != 0 && cfg->single_launch != 1) return FV2D_ERR_INVALID;
  if (cfg->band_rows != 0 && (cfg->band_rows < kMinBand || cfg->band_rows > 64)) return FV2D_ERR_INVALID;
  *out = nullptr;
  fv2d_server *s = new (std::nothrow) fv2d_server();
  if (!s) return FV2D_ERR_NOMEM;
  s->cfg = *cfg;
  s->t0 = std::chrono::steady_clock::now();
  s->device = cfg->device;
  if (cudaSetDevice(s->device) != cudaSuccess) {
    delete s;
    return FV2D_ERR_CUDA;
  }
  cudaDeviceGetAttribute(&s->num_sms, cudaDevAttrMultiProcessorCount, s->device);
  s->max_sims = cfg->max_sims;
  s->arena.budget = cfg->budget_bytes;
  bool ok = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) == cudaSuccess &&
            cudaMalloc(&s->d_sims, sizeof(SimDev) * s->max_sims) == cudaSuccess &&
            cudaMallocHost(&s->h_up, sizeof(SimDev) * s->max_sims) == cudaSuccess &&
            cudaMallocHost(&s->h_down, sizeof(SimDev) * s->max_sims) == cudaSuccess &&
            cudaMalloc(&s->d_tmaps, sizeof(CUtensorMap) * 2 * s->max_sims) == cudaSuccess &&
            cudaMallocHost(&s->h_tmaps, sizeof(CUtensorMap) * 2 * s->max_sims) == cudaSuccess &&
            cudaMalloc(&s->d_nwork, sizeof(int) * kLanes) == cudaSuccess &&
            cudaMallocHost(&s->h_nwork, sizeof(int) * kLanes) == cudaSuccess &&
            cudaMalloc(&s->d_cons, sizeof(double) * kConsBlocks * 8 * s->max_sims) == cudaSuccess &&
            cudaMalloc(&s->d_ctl, 2 * sizeof(unsigned int)) == cudaSuccess &&
            cudaMallocHost(&s->h_ctl, 2 * sizeof(unsigned int)) == cudaSuccess &&
            cudaMallocHost(&s->h_cons, sizeof(double) * kConsBlocks * 8 * s->max_sims) == cudaSuccess &&
            cudaEventCreate(&s->ev0) == cudaSuccess && cudaEventCreate(&s->ev1) == cudaSuccess &&
            cudaEventCreateWithFlags(&s->ev_fork, cudaEventDisableTiming) == cudaSuccess;
  for (int b = 0; ok && b < kLanes; ++b)
    ok = cudaStreamCreateWithFlags(&s->bstream[b], cudaStreamNonBlocking) == cudaSuccess &&
         cudaEventCreateWithFlags(&s->ev_join[b], cudaEventDisableTiming) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    fv2d_server_destroy(s);
    return FV2D_ERR_NOMEM;
  }
  std::memset(s->h_up, 0, sizeof(SimDev) * s->max_sims);
  cudaMemcpy(s->d_sims, s->h_up, sizeof(SimDev) * s->max_sims, cudaMemcpyHostToDevice);
  s->h_ctl[0] = 0u;
  s->h_ctl[1] = kTileWaitFinal;
  cudaMemcpy(s->d_ctl, s->h_ctl, 2 * sizeof(unsigned int), cudaMemcpyHostToDevice);
  std::memset(s->h_nwork, 0, sizeof(int) * kLanes);
  cudaMemcpy(s->d_nwork, s->h_nwork, sizeof(int) * kLanes, cudaMemcpyHostToDevice);
  s->slots.resize(s->max_sims);
  for (int k = s->max_sims - 1; k >= 0; --k) s->free_slots.push_back(k);
  s->cfg_grid.assign(num_cfgs(), 0);
  for (int c = 0; c < num_cfgs(); ++c) {
    int per_sm = 0;
    if (batch_setup(c, &per_sm) == cudaSuccess && per_sm > 0) s->cfg_grid[c] = per_sm * s->num_sms;
  }
  // the extended family: its first configuration that can run
  for (int c = 0; c < num_cfgs() && s->fam_cfg[FAM_EXT][0] < 0; ++c)
    if (((cfg_fams(c) >> FAM_EXT) & 1) && s->cfg_grid[c])
      for (int b = 0; b < kBuckets; ++b) s->fam_cfg[FAM_EXT][b] = c;
  // a forced configuration serves the families it has item bodies for; the
  // others keep their defaults
  const int forced = cfg->tile_config - 1;
  if (forced >= 0 && forced < num_cfgs() && s->cfg_grid[forced]) {
    for (int f = 0; f < kFamilies; ++f)
      if ((cfg_fams(forced) >> f) & 1)
        for (int b = 0; b < kBuckets; ++b) s->fam_cfg[f][b] = forced;
  } else if (cfg->autotune) {
    autotune(s);
  }
  if (cfg->single_launch)  // one configuration for a family's merged list: its largest grids'
    for (int f = 0; f < kFamilies; ++f)
      for (int b = 0; b < kBuckets - 1; ++b) s->fam_cfg[f][b] = s->fam_cfg[f][kBuckets - 1];
  if (s->fam_cfg[FAM_EXT][0] < 0) {  // no extended configuration can run on this device
    fv2d_server_destroy(s);
    return FV2D_ERR_CUDA;
  }
  publish_locked(s);  // no other thread yet
  s->worker = std::thread(worker_main, s);
  *out = s;
  return FV2D_OK;
}

int fv2d_server_destroy(fv2d_server *s) {
  if (!s) return FV2D_ERR_INVALID;
  s->stop.store(true);
  s->cv.notify_all();
  if (s->worker.joinable()) s->worker.join();
  if (s->stream) cudaStreamSynchronize(s->stream);
  for (auto &g : s->graphs) cudaGraphExecDestroy(g.second);
  s->arena.free_all();
  for (int b = 0; b < kLanes; ++b) {
    if (s->d_work[b]) cudaFree(s->d_work[b]);
    if (s->h_work[b]) cudaFreeHost(s->h_work[b]);
  }
  if (s->d_sims) cudaFree(s->d_sims);
  if (s->h_up) cudaFreeHost(s->h_up);
  if (s->h_down) cudaFreeHost(s->h_down);
  if (s->d_tmaps) cudaFree(s->d_tmaps);
  if (s->h_tmaps) cudaFreeHost(s->h_tmaps);
  if (s->d_nwork) cudaFree(s->d_nwork);
  if (s->h_nwork) cudaFreeHost(s->h_nwork);
  if (s->d_cons) cudaFree(s->d_cons);
  if (s->d_ctl) cudaFree(s->d_ctl);
  if (s->h_ctl) cudaFreeHost(s->h_ctl);
  if (s->h_cons) cudaFreeHost(s->h_cons);
  if (s->h_stage) cudaFreeHost(s->h_stage);
  if (s->ev0) cudaEventDestroy(s->ev0);
  if (s->ev1) cudaEventDestroy(s->ev1);
  if (s->ev_fork) cudaEventDestroy(s->ev_fork);
  for (int b = 0; b < kLanes; ++b) {
    if (s->ev_join[b]) cudaEventDestroy(s->ev_join[b]);
    if (s->bstream[b]) cudaStreamDestroy(s->bstream[b]);
  }
  if (s->stream) cudaStreamDestroy(s->stream);
  delete s;
  return FV2D_OK;
}

int fv2d_server_check_request(const fv2d_request *req, char *buf, int len) {
  if (!req || (len > 0 && !buf) || len < 0) return FV2D_ERR_INVALID;
  const char *why = check_request(*req);
  if (len > 0) std::snprintf(buf, (size_t)len, "%s", why ? why : "");
  return why ? FV2D_ERR_UNSUPPORTED : FV2D_OK;
}

int fv2d_server_submit(fv2d_server *s, const fv2d_request *req, int64_t *id) {
  if (!s || !req || !id) return FV2D_ERR_INVALID;
  if (check_request(*req)) return FV2D_ERR_UNSUPPORTED;
  int pitch;
  long long plane;
  size_t rows_off;
  if ((double)state_bytes(req->params, &pitch, &plane, &rows_off) > s->cfg.budget_bytes) return FV2D_ERR_SIZE;
  std::lock_guard<std::mutex> lock(s->mu);
  if (s->broken) return FV2D_ERR_STATE;
  Pending pd;
  pd.id = s->next_id++;
  pd.req = *req;
  pd.submit_s = s->now();
  s->queue.push_back(pd);
  s->n_submitted++;
  *id = pd.id;
  s->cv.notify_all();
  return FV2D_OK;
}

int fv2d_server_poll(fv2d_server *s, fv2d_result *out, int max, int *n) {
  if (!s || !n || max < 0 || (max > 0 && !out)) return FV2D_ERR_INVALID;
  std::lock_guard<std::mutex> lock(s->mu);
  const int k = std::min<int>(max, (int)s->done_unpolled.size());
  for (int i = 0; i < k; ++i) out[i] = s->done_unpolled[i];
  s->done_unpolled.erase(s->done_unpolled.begin(), s->done_unpolled.begin() + k);
  *n = k;
  return FV2D_OK;
}

int fv2d_server_drain(fv2d_server *s, double timeout_s) {
  if (!s || !(timeout_s >= 0)) return FV2D_ERR_INVALID;
  const double end = s->now() + timeout_s;
  std::unique_lock<std::mutex> lock(s->mu);
  for (;;) {
    if (s->broken) return s->fail_code;
    const bool idle = s->queue.empty() && (s->n_completed + s->n_failed) == s->n_submitted;
    if (idle) return FV2D_OK;
    if (s->now() > end) return FV2D_ERR_STATE;
    s->cv.wait_for(lock, std::chrono::milliseconds(5));
  }
}

int fv2d_server_get_prim(fv2d_server *s, int64_t id, double *q) {
  if (!s || !q) return FV2D_ERR_INVALID;
  std::shared_ptr<const Finished> held;  // keeps the state alive through a concurrent release
  {
    std::lock_guard<std::mutex> lock(s->mu);
    auto it = s->finished.find(id);
    if (it == s->finished.end()) return FV2D_ERR_STATE;
    held = it->second;
  }
  const Finished &f = *held;
  const size_t n = (size_t)f.res.Nx * f.res.Ny;
  const double gm1 = f.gamma - 1.0;
  for (size_t c = 0; c < n; ++c) {
    const double r = (double)f.U[c] + f.bg_r, mu = f.U[n + c], mv = f.U[2 * n + c],
                 E = (double)f.U[3 * n + c] + f.bg_e;
    const double u = mu / r, v = mv / r;
    q[4 * c] = r;
    q[4 * c + 1] = u;
    q[4 * c + 2] = v;
    q[4 * c + 3] = (E - 0.5 * r * (u * u + v * v)) * gm1;
  }
  return FV2D_OK;
}

int fv2d_server_release(fv2d_server *s, int64_t id) {
  if (!s) return FV2D_ERR_INVALID;
  std::lock_guard<std::mutex> lock(s->mu);
  return s->finished.erase(id) ? FV2D_OK : FV2D_ERR_STATE;
}

int fv2d_server_last_error(fv2d_server *s, char *buf, int len) {
  if (!s || !buf || len <= 0) return FV2D_ERR_INVALID;
  std::lock_guard<std::mutex> lock(s->mu);
  std::snprintf(buf, (size_t)len, "%s", s->err.c_str());
  return FV2D_OK;
}

int fv2d_server_inject_fault(fv2d_server *s) {
  if (!s) return FV2D_ERR_INVALID;
  s->inject.store(true);
  s->cv.notify_all();
  return FV2D_OK;
}

int fv2d_server_set_tile_wait_limit(fv2d_server *s, uint32_t polls) {
  if (!s) return FV2D_ERR_INVALID;
  s->wait_limit_req.store(polls == 0 ? UINT32_MAX : polls);
  s->cv.notify_all();
  return FV2D_OK;
}

int fv2d_server_get_stats(fv2d_server *s, fv2d_server_stats *out) {
  if (!s || !out) return FV2D_ERR_INVALID;
  std::lock_guard<std::mutex> lock(s->mu);
  std::memset(out, 0, sizeof(*out));
  // counters of the worker thread as it last published them
  out->submitted = s->n_submitted;
  out->admitted = s->pub.admitted;
  out->completed = s->n_completed;
  out->failed = s->n_failed;
  out->active = s->pub.active;
  out->queued = (int)s->queue.size();
  out->cell_updates = s->pub.cell_updates;
  out->busy_s = s->pub.busy_s;
  out->bytes_in_use = s->pub.bytes_in_use;
  out->bytes_reserved = s->pub.bytes_reserved;
  for (int b = 0; b < kBuckets; ++b) {
    out->bucket_cfg[b] = s->fam_cfg[FAM_PLAIN][b];
    out->diff_cfg[b] = s->fam_cfg[FAM_DIFF][b];
  }
  out->ext_cfg = s->fam_cfg[FAM_EXT][0];
  out->replays = s->pub.replays;
  return FV2D_OK;
}

}  // extern "C"
