// fv2d_api.cu -- C-ABI of the plain FP64 path (include/fv2d_gpu.h):
// context management, device buffers, TMA descriptors, the set-up / pack
// kernels and the launch sequence of the fused step.
//
// Device layout (per context): four field planes (rho, u, v, p) for each of
// the two primitive buffers and for the conservative state(s), each plane
// (Ny + 4) rows of `pitch` doubles (ghost ring of 2 included, pitch a multiple
// of 32 elements so that rows start on 256-byte boundaries).  Interior cell
// (i, j) lives at row j + 2, column i + 2, like the reference's
// Array(Nty, Ntx, 4) with Nghosts = 2.
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/fv2d_gpu.h"
#include "ic.h"
#include "problems.h"
#include "step_common.cuh"
#include "physics.cuh"
#include "nvtx_range.h"

namespace fv2d {
cudaError_t init_step_kernels();
cudaError_t launch_step(int rs, int recon, dim3 grid, cudaStream_t s, const CUtensorMap &t0, const CUtensorMap &t1,
                        const StepArgs &a);
cudaError_t launch_commit(cudaStream_t s, const StepArgs &a);
}

using namespace fv2d;

struct fv2d_ctx {
  fv2d_params p;
  int device = 0;
  cudaStream_t own_stream = nullptr, stream = nullptr;
  int pitch = 0;
  long long plane = 0;
  double *Q[2] = {nullptr, nullptr};
  double *U = nullptr, *U1 = nullptr;
  double *stage = nullptr;  // interleaved interior staging (Ny*Nx*4)
  // fv2d_prefetch_prim: a copy of the next input into `stage` on its own
  // stream, overlapping the work on `stream`
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t ev_stage_free = nullptr;  // recorded on `stream` after each of its uses of `stage`
  cudaEvent_t ev_prefetch = nullptr;    // recorded on copy_stream after the prefetch copy
  const double *prefetched = nullptr;   // host array the pending prefetch copies (null: none)
  float *grav_row = nullptr;
  double *kap_row = nullptr;
  double *log = nullptr;
  int log_cap = 0;
  DevState *st = nullptr;
  DevState *st_host = nullptr;  // page-locked mirror for readbacks
  bool st_fresh = false;        // st_host equals st: read back with no work queued since
  CUtensorMap tm[2];
  StepArgs args;
  double inv_tc = 0, inv_visc = 0;
  bool have_state = false;
  double *mirror_host = nullptr;  // caller's page-locked array registered by fv2d_set_host_mirror
  double *mirror_dev = nullptr;   // its device view
  bool mirror_valid = false;      // it holds the current state (written by the last fv2d_update)
  cudaGraphExec_t graph = nullptr;
  int graph_steps = 0;
  cudaStream_t graph_stream = nullptr;
  std::string err;
};

namespace {

thread_local std::string g_create_error;

int fail(fv2d_ctx *c, int code, const std::string &msg) {
  if (c) c->err = msg;
  return code;
}
int cuda_fail(fv2d_ctx *c, cudaError_t e, const char *what) {
  return fail(c, FV2D_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// The staging buffer is shared by the context's stream and the prefetch
// copy: before the stream uses it, a pending prefetch is waited for (and its
// data dropped); after the stream's use, an event tells the next prefetch
// when it may write.
void stage_take(fv2d_ctx *c) {
  if (c->prefetched) {
    cudaStreamWaitEvent(c->stream, c->ev_prefetch, 0);
    c->prefetched = nullptr;
  }
}
void stage_release(fv2d_ctx *c) { cudaEventRecord(c->ev_stage_free, c->stream); }
#define CK(call)                                              \
  do {                                                        \
    cudaError_t e_ = (call);                                  \
    if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call); \
  } while (0)

bool is_pow2_spacing(double d) {
  if (!(d > 0) || !std::isfinite(d)) return false;
  int e;
  double m = std::frexp(d, &e);
  return m == 0.5 && std::isfinite(1.0 / d);
}

PFN_cuTensorMapEncodeTiled_v12000 get_encode() {
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

// ------------------------------------------------------------------ kernels
__device__ __forceinline__ double ddiv_c(double x, double d, double inv_d, int pow2, uint64_t rw) {
  return pow2 ? x * inv_d : fv_div_by(x, d, rw);
}

// Set-up pass: interleaved interior primitives -> planes, every ghost cell
// from its source (BoundaryConditions.h:82-147), U = primToCons(Q)
// (SimInfo.h:589-600), and the inverse hyperbolic dt reduction
// (ComputeDt.h:26-52).  The last CTA stores dt for the next update.
__global__ void __launch_bounds__(256) prepare_kernel(PrepArgs a) {
  __shared__ double red[8];
  __shared__ int s_last;
  const long long n_int = (long long)a.Nx * a.Ny;
  const int W = a.Nx + 4;
  const long long n_ghost = 4LL * W + 4LL * a.Ny;
  const Gas<double> gas = make_gas(a.gamma, a.gm1, 1.0 / a.gm1, 0.0);
  double lmax = -1.0;
  // grid-stride over the interior cells and then the ghost cells: a few
  // thousand CTAs, so that the reduction's per-CTA atomics on the two state
  // words stay few
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < n_int + n_ghost;
       idx += (long long)gridDim.x * blockDim.x) {
  if (idx < n_int) {
    const int j = (int)(idx / a.Nx), i = (int)(idx % a.Nx);
    const double *s = a.q_aos + idx * 4;
    S4<double> q{s[0], s[1], s[2], s[3]};
    const long long g = (long long)(j + 2) * a.pitch + (i + 2);
    a.Q[g] = q.r;
    a.Q[a.plane + g] = q.u;
    a.Q[2 * a.plane + g] = q.v;
    a.Q[3 * a.plane + g] = q.p;
    S4<double> u = prim_to_cons(q, gas);
    a.U[g] = u.r;
    a.U[a.plane + g] = u.u;
    a.U[2 * a.plane + g] = u.v;
    a.U[3 * a.plane + g] = u.p;
    const double cs = sound_speed(q, gas);
    const double ih = ddiv_c(cs + fabs(q.u), a.dx, a.inv_dx, a.dx_pow2, a.rw_dx) +
                      ddiv_c(cs + fabs(q.v), a.dy, a.inv_dy, a.dy_pow2, a.rw_dy);
    lmax = fmax(lmax, ih);
  } else if (idx < n_int + n_ghost) {
    long long k = idx - n_int;
    int px, py;  // padded coordinates of the ghost cell
    if (k < 4LL * W) {
      const int r = (int)(k / W);
      px = (int)(k % W);
      py = (r < 2) ? r : a.Ny + r;  // rows 0,1 and Ny+2, Ny+3
    } else {
      k -= 4LL * W;
      const int c = (int)(k / a.Ny);
      py = (int)(k % a.Ny) + 2;
      px = (c < 2) ? c : a.Nx + c;  // columns 0,1 and Nx+2, Nx+3
    }
    int sx = px - 2, sy = py - 2;
    bool nx = false, ny = false;
    if (sx < 0 || sx >= a.Nx) sx = ghost_source(sx, a.Nx, a.bcx, &nx);
    if (sy < 0 || sy >= a.Ny) sy = ghost_source(sy, a.Ny, a.bcy, &ny);
    const double *s = a.q_aos + ((long long)sy * a.Nx + sx) * 4;
    const long long g = (long long)py * a.pitch + px;
    a.Q[g] = s[0];
    a.Q[a.plane + g] = nx ? s[1] * -1.0 : s[1];
    a.Q[2 * a.plane + g] = ny ? s[2] * -1.0 : s[2];
    a.Q[3 * a.plane + g] = s[3];
  }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) lmax = fmax(lmax, __shfl_xor_sync(0xffffffffu, lmax, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = lmax;
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = -1.0;
    for (int w = 0; w < 8; ++w) m = fmax(m, red[w]);
    if (m >= 0.0) atomicMax(&a.st->acc_hyp, (unsigned long long)__double_as_longlong(m));
    __threadfence();
    s_last = (atomicAdd(&a.st->ticket, 1u) == (unsigned)a.nblocks - 1u);
  }
  __syncthreads();
  if (!s_last || threadIdx.x != 0) return;
  __threadfence();
  volatile DevState *vs = a.st;
  const double inv_hyp = __longlong_as_double((long long)atomicAdd(&a.st->acc_hyp, 0ull));
  double m = inv_hyp;
  if (m < a.inv_tc) m = a.inv_tc;
  if (m < a.inv_visc) m = a.inv_visc;
  vs->inv_hyp = inv_hyp;
  vs->dt = a.CFL / m;
  for (int k = 0; k < 3; ++k) {
    vs->counters[k] = 0ull;
    vs->cnt_acc[k] = 0ull;
  }
  a.st->acc_hyp = 0ull;
  __threadfence();
  a.st->ticket = 0u;
}

// Planes (interior) -> interleaved array.
__global__ void pack_kernel(const double *P, long long plane, int pitch, int Nx, int Ny, double *out) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)Nx * Ny) return;
  const int j = (int)(idx / Nx), i = (int)(idx % Nx);
  const long long g = (long long)(j + 2) * pitch + (i + 2);
  double *o = out + idx * 4;
  o[0] = P[g];
  o[1] = P[plane + g];
  o[2] = P[2 * plane + g];
  o[3] = P[3 * plane + g];
}

// Loop control of fv2d_advance, evaluated before its first iteration
// (main.cpp:62-64).
__global__ void begin_kernel(DevState *st, double tend, double next_save, double eps, int check_save,
                             int skip_first, int max_steps) {
  st->tend = tend;
  st->next_save = next_save;
  st->eps = eps;
  st->check_save = check_save;
  st->max_steps = max_steps;
  st->steps_in_call = 0;
  const double t = st->t;
  int s = RUN_RUNNING;
  if (!(t + eps < tend))
    s = RUN_DONE;
  else if (check_save && !skip_first && t + eps > next_save)
    s = RUN_SAVE;
  else if (!(st->dt > 0.0) || isnan(st->dt) || isinf(st->dt))
    s = RUN_NUMERIC;
  else if (max_steps <= 0)
    s = RUN_PAUSED;
  st->status = s;
}

int sync_state(fv2d_ctx *ctx) {
  CK(cudaMemcpyAsync(ctx->st_host, ctx->st, sizeof(DevState), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->st_fresh = true;
  return FV2D_OK;
}
// The device state as the host last read it, read again only when work has
// been queued since (a set_prim followed by compute_dt needs one round trip).
int fresh_state(fv2d_ctx *ctx) { return ctx->st_fresh ? FV2D_OK : sync_state(ctx); }

void fill_args(fv2d_ctx *c) {
  const fv2d_params &p = c->p;
  StepArgs &a = c->args;
  std::memset(&a, 0, sizeof(a));
  a.Q[0] = c->Q[0];
  a.Q[1] = c->Q[1];
  a.U = c->U;
  a.U1 = c->U1;
  a.grav_row = c->grav_row;
  a.kap_row = c->kap_row;
  a.st = c->st;
  a.log = c->log;
  a.plane = c->plane;
  a.pitch = c->pitch;
  a.Nx = p.Nx;
  a.Ny = p.Ny;
  const int gx = (p.Nx + TX - 1) / TX, gy = (p.Ny + TY - 1) / TY;
  a.nblocks = gx * gy;
  a.gamma = p.gamma0;
  a.gm1 = p.gamma0 - 1.0;
  a.entho = 1.0 / (p.gamma0 - 1.0);
  a.fslp_K = p.fslp_K;
  a.dx = (p.xmax - p.xmin) / p.Nx;  // SimInfo.h:375-376
  a.dy = (p.ymax - p.ymin) / p.Ny;
  a.dx_pow2 = is_pow2_spacing(a.dx);
  a.dy_pow2 = is_pow2_spacing(a.dy);
  a.inv_dx = a.dx_pow2 ? 1.0 / a.dx : 0.0;
  a.inv_dy = a.dy_pow2 ? 1.0 / a.dy : 0.0;
  a.rw_dx = softfp::recip_of_host(a.dx);
  a.rw_dy = softfp::recip_of_host(a.dy);
  a.one_over_dx = 1.0 / a.dx;
  a.one_over_dy = 1.0 / a.dy;
  a.gx_dx = p.gx * a.dx;
  a.gy_dy = p.gy * a.dy;
  a.gxf = (double)(float)p.gx;
  a.gyf = (double)(float)p.gy;
  a.eps_reset = p.epsilon_reset_negative;
  a.CFL = p.CFL;
  a.inv_tc = c->inv_tc;
  a.inv_visc = c->inv_visc;
  a.mu = p.mu;
  a.bctc_ymin_value = p.bctc_ymin_value;
  a.bctc_ymax_value = p.bctc_ymax_value;
  a.bcx = p.boundary_x;
  a.bcy = p.boundary_y;
  a.grav_mode = p.gravity_mode;
  a.tc = p.thermal_conductivity_active ? 1 : 0;
  a.visc = p.viscosity_active ? 1 : 0;
  a.wb = p.well_balanced_flux_at_y_bc ? 1 : 0;
  a.bctc_ymin = p.bctc_ymin;
  a.bctc_ymax = p.bctc_ymax;
}

int recon_kind(int r) {
  if (r == FV2D_PLM) return RECON_PLM;
  if (r == FV2D_MUSCL_HANCOCK) return RECON_MH;
  return RECON_PCM;  // PCM and PCM_WB (Update.h:27-33 falls through to PCM)
}

int launch_update(fv2d_ctx *ctx, int driven, double dt) {
  ctx->st_fresh = false;
  StepArgs a = ctx->args;
  a.driven = driven;
  a.dt_arg = dt;
  a.mirror = driven ? nullptr : ctx->mirror_dev;  // captured device loops never write it
  const dim3 grid((ctx->p.Nx + TX - 1) / TX, (ctx->p.Ny + TY - 1) / TY);
  const int rk = recon_kind(ctx->p.reconstruction);
  if (ctx->p.time_stepping == FV2D_TS_EULER) {
    a.stage = STAGE_EULER;
    CK(launch_step(ctx->p.riemann_solver, rk, grid, ctx->stream, ctx->tm[0], ctx->tm[1], a));
  } else {
    a.stage = STAGE_RK2_PREDICT;
    CK(launch_step(ctx->p.riemann_solver, rk, grid, ctx->stream, ctx->tm[0], ctx->tm[1], a));
    a.stage = STAGE_RK2_CORRECT;
    CK(launch_step(ctx->p.riemann_solver, rk, grid, ctx->stream, ctx->tm[0], ctx->tm[1], a));
  }
  CK(launch_commit(ctx->stream, a));
  return FV2D_OK;
}

// Device view of a page-locked (or registered) host array, or null when the
// pointer is ordinary pageable memory.
const double *mapped_host(const double *p) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (at.type != cudaMemoryTypeHost || !at.devicePointer) return nullptr;
  return static_cast<const double *>(at.devicePointer);
}

int run_prepare(fv2d_ctx *ctx, const double *src) {
  const fv2d_params &p = ctx->p;
  if (int rc = fresh_state(ctx)) return rc;  // the parity of the current buffer
  ctx->mirror_valid = false;
  PrepArgs pa;
  std::memset(&pa, 0, sizeof(pa));
  pa.q_aos = src;
  pa.Q = ctx->Q[ctx->st_host->parity];
  pa.U = ctx->U;
  pa.st = ctx->st;
  pa.plane = ctx->plane;
  pa.pitch = ctx->pitch;
  pa.Nx = p.Nx;
  pa.Ny = p.Ny;
  const long long n = (long long)p.Nx * p.Ny + 4LL * (p.Nx + 4) + 4LL * p.Ny;
  const int nb = (int)std::min<long long>((n + 255) / 256, 8LL * 152);
  pa.nblocks = nb;
  pa.gamma = ctx->args.gamma;
  pa.gm1 = ctx->args.gm1;
  pa.dx = ctx->args.dx;
  pa.dy = ctx->args.dy;
  pa.inv_dx = ctx->args.inv_dx;
  pa.inv_dy = ctx->args.inv_dy;
  pa.dx_pow2 = ctx->args.dx_pow2;
  pa.dy_pow2 = ctx->args.dy_pow2;
  pa.rw_dx = ctx->args.rw_dx;
  pa.rw_dy = ctx->args.rw_dy;
  pa.CFL = p.CFL;
  pa.inv_tc = ctx->inv_tc;
  pa.inv_visc = ctx->inv_visc;
  pa.bcx = p.boundary_x;
  pa.bcy = p.boundary_y;
  ctx->st_fresh = false;
  prepare_kernel<<<nb, 256, 0, ctx->stream>>>(pa);
  CK(cudaGetLastError());
  ctx->have_state = true;
  return FV2D_OK;
}

int encode_maps(fv2d_ctx *ctx) {
  PFN_cuTensorMapEncodeTiled_v12000 enc = get_encode();
  if (!enc) return fail(ctx, FV2D_ERR_CUDA, "cuTensorMapEncodeTiled entry point not available");
  const fv2d_params &p = ctx->p;
  for (int b = 0; b < 2; ++b) {
    cuuint64_t dims[3] = {(cuuint64_t)(p.Nx + 4), (cuuint64_t)(p.Ny + 4), 4};
    cuuint64_t strides[2] = {(cuuint64_t)ctx->pitch * sizeof(double), (cuuint64_t)ctx->plane * sizeof(double)};
    cuuint32_t box[3] = {(cuuint32_t)SW, (cuuint32_t)SH, 4};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = enc(&ctx->tm[b], CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, ctx->Q[b], dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(ctx, FV2D_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
  }
  return FV2D_OK;
}

// Launch-bound loops are replayed from a CUDA graph of G fused steps; every
// step reads its dt, buffer parity and stop flag from device memory, so one
// captured sequence serves every replay and steps after a stop are no-ops.
int ensure_graph(fv2d_ctx *ctx) {
  const int G = 32;
  if (ctx->graph && ctx->graph_stream == ctx->stream) return FV2D_OK;
  if (ctx->graph) {
    cudaGraphExecDestroy(ctx->graph);
    ctx->graph = nullptr;
  }
  cudaGraph_t g;
  CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  int rc = FV2D_OK;
  for (int k = 0; k < G && rc == FV2D_OK; ++k) rc = launch_update(ctx, 1, 0.0);
  cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
  if (rc) return rc;
  if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaStreamEndCapture");
  e = cudaGraphInstantiate(&ctx->graph, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaGraphInstantiate");
  ctx->graph_stream = ctx->stream;
  ctx->graph_steps = G;
  return FV2D_OK;
}

void free_all(fv2d_ctx *c) {
  if (c->copy_stream) cudaStreamSynchronize(c->copy_stream);
  if (c->ev_stage_free) cudaEventDestroy(c->ev_stage_free);
  if (c->ev_prefetch) cudaEventDestroy(c->ev_prefetch);
  if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
  if (c->graph) cudaGraphExecDestroy(c->graph);
  for (double *ptr : {c->Q[0], c->Q[1], c->U, c->U1, c->stage, c->kap_row, c->log})
    if (ptr) cudaFree(ptr);
  if (c->grav_row) cudaFree(c->grav_row);
  if (c->st) cudaFree(c->st);
  if (c->st_host) cudaFreeHost(c->st_host);
  if (c->own_stream) cudaStreamDestroy(c->own_stream);
}

}  // namespace

extern "C" {

void fv2d_params_default(fv2d_params *p) {
  if (p) params_default(p);
}

size_t fv2d_params_size(void) { return sizeof(fv2d_params); }

const char *fv2d_last_error(fv2d_ctx *ctx) {
  if (!ctx) return g_create_error.c_str();
  return ctx->err.c_str();
}

int fv2d_build_info(char *buf, int len) {
  if (!buf || len <= 0) return FV2D_ERR_INVALID;
  std::snprintf(buf, (size_t)len, "fv2d_gpu fp64 step: tile %dx%d, %d threads/CTA, halo %d, sm_103a, TMA 3-D box %dx%dx4",
                TX, TY, NT, HALO, SW, SH);
  return FV2D_OK;
}

int fv2d_create(const fv2d_params *p, int device, fv2d_ctx **out) {
  g_create_error.clear();
  if (!p || !out) {
    g_create_error = "null argument";
    return FV2D_ERR_INVALID;
  }
  *out = nullptr;
  if (const char *why = validate(*p)) {
    g_create_error = why;
    return FV2D_ERR_INVALID;
  }
  fv2d_ctx *ctx = new (std::nothrow) fv2d_ctx();
  if (!ctx) return FV2D_ERR_NOMEM;
  ctx->p = *p;
  auto bail = [&](int code) {
    g_create_error = ctx->err;
    free_all(ctx);
    delete ctx;
    return code;
  };
  cudaError_t e;
  if (device >= 0) {
    if ((e = cudaSetDevice(device)) != cudaSuccess) return bail(cuda_fail(ctx, e, "cudaSetDevice"));
  }
  cudaGetDevice(&ctx->device);
  if ((e = init_step_kernels()) != cudaSuccess) return bail(cuda_fail(ctx, e, "step kernel attributes"));
  if ((e = cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking)) != cudaSuccess ||
      (e = cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking)) != cudaSuccess ||
      (e = cudaEventCreateWithFlags(&ctx->ev_stage_free, cudaEventDisableTiming)) != cudaSuccess ||
      (e = cudaEventCreateWithFlags(&ctx->ev_prefetch, cudaEventDisableTiming)) != cudaSuccess)
    return bail(cuda_fail(ctx, e, "cudaStreamCreate"));
  ctx->stream = ctx->own_stream;

  const int W = p->Nx + 4, H = p->Ny + 4;
  ctx->pitch = (W + 31) / 32 * 32;
  ctx->plane = (long long)H * ctx->pitch;
  const size_t bytes = sizeof(double) * 4 * (size_t)ctx->plane;
  const size_t nint = (size_t)p->Nx * p->Ny;
  bool ok = cudaMalloc(&ctx->Q[0], bytes) == cudaSuccess && cudaMalloc(&ctx->Q[1], bytes) == cudaSuccess &&
            cudaMalloc(&ctx->U, bytes) == cudaSuccess &&
            (p->time_stepping != FV2D_TS_RK2 || cudaMalloc(&ctx->U1, bytes) == cudaSuccess) &&
            cudaMalloc(&ctx->stage, sizeof(double) * 4 * nint) == cudaSuccess &&
            cudaMalloc(&ctx->grav_row, sizeof(float) * p->Ny) == cudaSuccess &&
            cudaMalloc(&ctx->kap_row, sizeof(double) * 4 * p->Ny) == cudaSuccess &&
            cudaMalloc(&ctx->st, sizeof(DevState)) == cudaSuccess &&
            cudaMallocHost(&ctx->st_host, sizeof(DevState)) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    ctx->err = "device allocation failed";
    return bail(FV2D_ERR_NOMEM);
  }
  ctx->log_cap = 4096;
  if (cudaMalloc(&ctx->log, sizeof(double) * 6 * ctx->log_cap) != cudaSuccess) {
    cudaGetLastError();
    ctx->err = "device allocation failed";
    return bail(FV2D_ERR_NOMEM);
  }
  // zero everything once: ghosts of never-written buffers stay finite
  for (double *ptr : {ctx->Q[0], ctx->Q[1], ctx->U})
    cudaMemsetAsync(ptr, 0, bytes, ctx->stream);
  if (ctx->U1) cudaMemsetAsync(ctx->U1, 0, bytes, ctx->stream);

  // position-only tables, computed on the host like the reference's CPU build
  std::vector<float> grow;
  std::vector<double> krow;
  try {
    grow.resize(p->Ny);
    krow.resize(4 * (size_t)p->Ny);
  } catch (const std::bad_alloc &) {
    ctx->err = "host allocation failed";
    return bail(FV2D_ERR_NOMEM);
  }
  for (int j = 0; j < p->Ny; ++j) {
    grow[j] = (p->gravity_mode == FV2D_GRAV_ANALYTICAL) ? analytical_gravity_row(*p, j) : 0.0f;
    kappa_row(*p, j, &krow[4 * (size_t)j]);
  }
  parabolic_inv_dt(*p, &ctx->inv_tc, &ctx->inv_visc);
  if ((e = cudaMemcpy(ctx->grav_row, grow.data(), sizeof(float) * p->Ny, cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemcpy(ctx->kap_row, krow.data(), sizeof(double) * 4 * p->Ny, cudaMemcpyHostToDevice)) != cudaSuccess)
    return bail(cuda_fail(ctx, e, "cudaMemcpy tables"));

  DevState s0;
  std::memset(&s0, 0, sizeof(s0));
  s0.status = RUN_PAUSED;
  s0.log_cap = ctx->log_cap;
  if ((e = cudaMemcpy(ctx->st, &s0, sizeof(s0), cudaMemcpyHostToDevice)) != cudaSuccess)
    return bail(cuda_fail(ctx, e, "cudaMemcpy state"));
  if (int rc = encode_maps(ctx)) return bail(rc);
  fill_args(ctx);
  if ((e = cudaStreamSynchronize(ctx->stream)) != cudaSuccess) return bail(cuda_fail(ctx, e, "set-up"));
  *out = ctx;
  return FV2D_OK;
}

int fv2d_destroy(fv2d_ctx *ctx) {
  if (!ctx) return FV2D_ERR_INVALID;
  cudaStreamSynchronize(ctx->stream);
  free_all(ctx);
  delete ctx;
  return FV2D_OK;
}

int fv2d_set_stream(fv2d_ctx *ctx, void *stream) {
  if (!ctx) return FV2D_ERR_INVALID;
  ctx->stream = stream ? static_cast<cudaStream_t>(stream) : ctx->own_stream;
  return FV2D_OK;
}

int fv2d_set_prim_device(fv2d_ctx *ctx, const double *q_dev) {
  if (!ctx || !q_dev) return FV2D_ERR_INVALID;
  const size_t n = (size_t)ctx->p.Nx * ctx->p.Ny * 4;
  stage_take(ctx);
  CK(cudaMemcpyAsync(ctx->stage, q_dev, n * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
  const int rc = run_prepare(ctx, ctx->stage);
  stage_release(ctx);
  return rc;
}

int fv2d_set_prim(fv2d_ctx *ctx, const double *q_host) {
  const fv2d::NvtxRange nvtx_range("fv2d_set_prim");
  if (!ctx || !q_host) return FV2D_ERR_INVALID;
  // A prefetched copy of q_host (fv2d_prefetch_prim) is converted from the
  // staging buffer.  Otherwise page-locked host memory is read by the set-up
  // kernel itself over the host link (one pass instead of a copy then a
  // pass); pageable memory is copied to the staging buffer first.
  const double *src = nullptr;
  bool staged = false;
  if (ctx->prefetched == q_host) {
    CK(cudaStreamWaitEvent(ctx->stream, ctx->ev_prefetch, 0));
    ctx->prefetched = nullptr;
    src = ctx->stage;
    staged = true;
  } else if (!(src = mapped_host(q_host))) {
    const size_t n = (size_t)ctx->p.Nx * ctx->p.Ny * 4;
    stage_take(ctx);
    CK(cudaMemcpyAsync(ctx->stage, q_host, n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    src = ctx->stage;
    staged = true;
  }
  const int rc = run_prepare(ctx, src);
  if (staged) stage_release(ctx);
  if (rc) return rc;
  return sync_state(ctx);  // q_host may be reused on return; the new dt is read back with it
}

int fv2d_prefetch_prim(fv2d_ctx *ctx, const double *q_host) {
  const fv2d::NvtxRange nvtx_range("fv2d_prefetch_prim");
  if (!ctx || !q_host) return FV2D_ERR_INVALID;
  if (!mapped_host(q_host)) return fail(ctx, FV2D_ERR_INVALID, "prefetch needs page-locked host memory");
  const size_t n = (size_t)ctx->p.Nx * ctx->p.Ny * 4;
  // after the stream's last use of the staging buffer (not after the rest of
  // its queued work: the copy overlaps a step in flight)
  CK(cudaStreamWaitEvent(ctx->copy_stream, ctx->ev_stage_free, 0));
  CK(cudaMemcpyAsync(ctx->stage, q_host, n * sizeof(double), cudaMemcpyHostToDevice, ctx->copy_stream));
  CK(cudaEventRecord(ctx->ev_prefetch, ctx->copy_stream));
  ctx->prefetched = q_host;
  return FV2D_OK;
}

int fv2d_set_host_mirror(fv2d_ctx *ctx, double *q_host) {
  if (!ctx) return FV2D_ERR_INVALID;
  CK(cudaStreamSynchronize(ctx->stream));  // no step in flight writes the old array
  ctx->mirror_host = nullptr;
  ctx->mirror_dev = nullptr;
  ctx->mirror_valid = false;
  if (!q_host) return FV2D_OK;
  const double *dev = mapped_host(q_host);
  if (!dev) return fail(ctx, FV2D_ERR_INVALID, "host mirror must be page-locked (cudaHostAlloc / cudaHostRegister)");
  if ((reinterpret_cast<uintptr_t>(q_host) | reinterpret_cast<uintptr_t>(dev)) & 15)
    return fail(ctx, FV2D_ERR_INVALID, "host mirror must be 16-byte aligned");
  ctx->mirror_host = q_host;
  ctx->mirror_dev = const_cast<double *>(dev);
  return FV2D_OK;
}

int fv2d_init_problem(fv2d_ctx *ctx, int problem) {
  const fv2d::NvtxRange nvtx_range("fv2d_init_problem");
  if (!ctx) return FV2D_ERR_INVALID;
  if (!problem_valid(problem)) return fail(ctx, FV2D_ERR_INVALID, "unknown problem id");
  const fv2d_params &p = ctx->p;
  std::vector<double> q;
  try {
    q.resize((size_t)p.Nx * p.Ny * 4);
  } catch (const std::bad_alloc &) {
    return fail(ctx, FV2D_ERR_NOMEM, "host allocation failed");
  }
  for (int j = 0; j < p.Ny; ++j)
    for (int i = 0; i < p.Nx; ++i) init_cell(p, problem, i, j, &q[((size_t)j * p.Nx + i) * 4]);
  stage_take(ctx);
  CK(cudaMemcpyAsync(ctx->stage, q.data(), q.size() * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  int rc = run_prepare(ctx, ctx->stage);
  stage_release(ctx);
  if (rc) return rc;
  CK(cudaStreamSynchronize(ctx->stream));  // q is a local buffer
  return FV2D_OK;
}

static int get_planes(fv2d_ctx *ctx, const double *planes, double *dst, cudaMemcpyKind kind) {
  const fv2d_params &p = ctx->p;
  const long long n = (long long)p.Nx * p.Ny;
  stage_take(ctx);
  pack_kernel<<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>(planes, ctx->plane, ctx->pitch, p.Nx, p.Ny,
                                                                     ctx->stage);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(dst, ctx->stage, (size_t)n * 4 * sizeof(double), kind, ctx->stream));
  stage_release(ctx);
  CK(cudaStreamSynchronize(ctx->stream));
  return FV2D_OK;
}

int fv2d_get_prim(fv2d_ctx *ctx, double *q_host) {
  const fv2d::NvtxRange nvtx_range("fv2d_get_prim");
  if (!ctx || !q_host) return FV2D_ERR_INVALID;
  if (!ctx->have_state) return fail(ctx, FV2D_ERR_STATE, "no state: call set_prim or init_problem first");
  if (int rc = sync_state(ctx)) return rc;
  if (ctx->mirror_valid && q_host == ctx->mirror_host) return FV2D_OK;  // the last update wrote it
  return get_planes(ctx, ctx->Q[ctx->st_host->parity], q_host, cudaMemcpyDeviceToHost);
}

int fv2d_get_prim_device(fv2d_ctx *ctx, double *q_dev) {
  if (!ctx || !q_dev) return FV2D_ERR_INVALID;
  if (!ctx->have_state) return fail(ctx, FV2D_ERR_STATE, "no state: call set_prim or init_problem first");
  if (int rc = sync_state(ctx)) return rc;
  return get_planes(ctx, ctx->Q[ctx->st_host->parity], q_dev, cudaMemcpyDeviceToDevice);
}

int fv2d_get_cons(fv2d_ctx *ctx, double *u_host) {
  if (!ctx || !u_host) return FV2D_ERR_INVALID;
  if (!ctx->have_state) return fail(ctx, FV2D_ERR_STATE, "no state: call set_prim or init_problem first");
  return get_planes(ctx, ctx->U, u_host, cudaMemcpyDeviceToHost);
}

int fv2d_compute_dt(fv2d_ctx *ctx, double *dt, double *inv_hyp, double *inv_tc, double *inv_visc) {
  const fv2d::NvtxRange nvtx_range("fv2d_compute_dt");
  if (!ctx) return FV2D_ERR_INVALID;
  if (!ctx->have_state) return fail(ctx, FV2D_ERR_STATE, "no state: call set_prim or init_problem first");
  if (int rc = fresh_state(ctx)) return rc;
  if (dt) *dt = ctx->st_host->dt;
  if (inv_hyp) *inv_hyp = ctx->st_host->inv_hyp;
  if (inv_tc) *inv_tc = ctx->inv_tc;
  if (inv_visc) *inv_visc = ctx->inv_visc;
  return FV2D_OK;
}

int fv2d_update(fv2d_ctx *ctx, double dt) {
  const fv2d::NvtxRange nvtx_range("fv2d_update");
  if (!ctx) return FV2D_ERR_INVALID;
  if (!ctx->have_state) return fail(ctx, FV2D_ERR_STATE, "no state: call set_prim or init_problem first");
  ctx->mirror_valid = false;
  if (int rc = launch_update(ctx, 0, dt)) return rc;
  ctx->mirror_valid = ctx->mirror_dev != nullptr;
  return FV2D_OK;
}

int fv2d_get_device_errors(fv2d_ctx *ctx, int *bits) {
  if (!ctx || !bits) return FV2D_ERR_INVALID;
  if (int rc = sync_state(ctx)) return rc;
  *bits = ctx->st_host->error;
  return FV2D_OK;
}

int fv2d_get_counters(fv2d_ctx *ctx, uint64_t out[3]) {
  if (!ctx || !out) return FV2D_ERR_INVALID;
  if (int rc = sync_state(ctx)) return rc;
  for (int k = 0; k < 3; ++k) out[k] = ctx->st_host->counters[k];
  return FV2D_OK;
}

int fv2d_get_time(fv2d_ctx *ctx, double *t, int *iteration) {
  if (!ctx) return FV2D_ERR_INVALID;
  if (int rc = sync_state(ctx)) return rc;
  if (t) *t = ctx->st_host->t;
  if (iteration) *iteration = ctx->st_host->ite;
  return FV2D_OK;
}

int fv2d_set_time(fv2d_ctx *ctx, double t, int iteration) {
  if (!ctx) return FV2D_ERR_INVALID;
  if (int rc = sync_state(ctx)) return rc;
  ctx->st_host->t = t;
  ctx->st_host->ite = iteration;
  CK(cudaMemcpyAsync(ctx->st, ctx->st_host, sizeof(DevState), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return FV2D_OK;
}

int fv2d_advance(fv2d_ctx *ctx, int max_steps, double tend, double next_save, int skip_first_save_check, double *t,
                 int *steps_done, int *status) {
  const fv2d::NvtxRange nvtx_range("fv2d_advance");
  if (!ctx) return FV2D_ERR_INVALID;
  if (!ctx->have_state) return fail(ctx, FV2D_ERR_STATE, "no state: call set_prim or init_problem first");
  if (max_steps < 0) return fail(ctx, FV2D_ERR_INVALID, "max_steps < 0");
  ctx->mirror_valid = false;
  ctx->st_fresh = false;
  const int check_save = next_save >= 0.0 ? 1 : 0;
  begin_kernel<<<1, 1, 0, ctx->stream>>>(ctx->st, tend, next_save, ctx->p.epsilon, check_save,
                                         skip_first_save_check, max_steps);
  CK(cudaGetLastError());
  if (int rc = ensure_graph(ctx)) return rc;
  const int G = ctx->graph_steps;
  long long launched = 0;  // no overflow for max_steps near INT_MAX
  for (;;) {
    // keep a few replays in flight between status checks
    const int burst = 4;
    for (int b = 0; b < burst && launched < max_steps; ++b) {
      CK(cudaGraphLaunch(ctx->graph, ctx->stream));
      launched += G;
    }
    if (int rc = sync_state(ctx)) return rc;
    if (ctx->st_host->status != RUN_RUNNING || launched >= max_steps) break;
  }
  const DevState &s = *ctx->st_host;
  if (t) *t = s.t;
  if (steps_done) *steps_done = s.steps_in_call;
  int out = FV2D_RUN_STEPS;
  if (s.status == RUN_DONE) out = FV2D_RUN_DONE;
  else if (s.status == RUN_SAVE) out = FV2D_RUN_SAVE;
  else if (s.status == RUN_NUMERIC) out = FV2D_RUN_NUMERIC;
  if (status) *status = out;
  if (s.error) return fail(ctx, FV2D_ERR_CUDA, "a step kernel timed out waiting for its tile load");
  return out == FV2D_RUN_NUMERIC ? fail(ctx, FV2D_ERR_NUMERIC, "non-finite or non-positive dt") : FV2D_OK;
}

int fv2d_run_async(fv2d_ctx *ctx, int n) {
  const fv2d::NvtxRange nvtx_range("fv2d_run_async");
  if (!ctx || n < 0) return FV2D_ERR_INVALID;
  if (!ctx->have_state) return fail(ctx, FV2D_ERR_STATE, "no state: call set_prim or init_problem first");
  ctx->mirror_valid = false;
  ctx->st_fresh = false;
  begin_kernel<<<1, 1, 0, ctx->stream>>>(ctx->st, INFINITY, -1.0, ctx->p.epsilon, 0, 1, n);
  CK(cudaGetLastError());
  if (int rc = ensure_graph(ctx)) return rc;
  long long k = 0;
  for (; k + ctx->graph_steps <= n; k += ctx->graph_steps) CK(cudaGraphLaunch(ctx->graph, ctx->stream));
  for (; k < n; ++k)
    if (int rc = launch_update(ctx, 1, 0.0)) return rc;
  return FV2D_OK;
}

int fv2d_get_step_log(fv2d_ctx *ctx, double *records, int max_records, int *count) {
  if (!ctx || !records || max_records < 0) return FV2D_ERR_INVALID;
  if (int rc = sync_state(ctx)) return rc;
  int n = std::min(std::min(ctx->st_host->steps_in_call, ctx->log_cap), max_records);
  if (n > 0) {
    CK(cudaMemcpyAsync(records, ctx->log, sizeof(double) * 6 * n, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
  }
  if (count) *count = n;
  return FV2D_OK;
}

}  // extern "C"
