// noalloc.cu -- CFL time step of a caller-owned primitive array without any
// device allocation (fv2d_compute_dt_noalloc in include/fv2d_gpu.h).
//
// Who needs this: callers that cannot call cudaMalloc -- code whose device
// memory is owned by another allocator (a framework memory pool that must
// account for every byte, or a process that reserved all device memory up
// front), and loops that cannot afford the device-wide synchronisation an
// allocation may cause.  They pass their own input and output arrays; the
// only scratch the reduction needs lives in a fixed array inside this
// library's device code.  CUDA loads a library's device code lazily by default:
// the first call on a device loads this module there (which may allocate
// device memory and synchronise, like any first use of a module) and looks up
// the array's address; every later call allocates nothing.  Callers whose
// loop must not allocate make one call before it (and before any stream
// capture).
//
// The scratch: one static array of 4096 per-CTA partial maxima plus a
// completion ticket (32 KB + 256 B, resident on every GPU that loads the
// library until the process exits).  One CTA handles
// FV2D_NOALLOC_CELLS_PER_BLOCK cells, which bounds a grid at
// FV2D_NOALLOC_MAX_CELLS cells (a 4096 x 4096 grid); larger grids are
// rejected with FV2D_ERR_SIZE before any GPU work.  Every call uses the same
// array and leaves its contents behind; the ticket is cleared at the start of
// each call.  Two calls whose work overlaps on the GPU (different streams, or
// different host threads) race on the array: serialise them.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>

#include "../../include/fv2d_gpu.h"
#include "physics.cuh"
#include "problems.h"

namespace {

constexpr int kThreads = 256;
constexpr int kCellsPerThread = 16;
constexpr int kCellsPerBlock = kThreads * kCellsPerThread;  // FV2D_NOALLOC_CELLS_PER_BLOCK
constexpr int kMaxBlocks = FV2D_NOALLOC_MAX_CELLS / kCellsPerBlock;
constexpr int kTicketSlot = kMaxBlocks;  // after the partials, own 256-byte line
constexpr int kScratchWords = kMaxBlocks + 32;

static_assert(kCellsPerBlock == FV2D_NOALLOC_CELLS_PER_BLOCK, "cells per CTA");
static_assert((long long)kMaxBlocks * kCellsPerBlock == FV2D_NOALLOC_MAX_CELLS, "grid bound");

// Per-CTA partial maxima (bits of the CTA's maximum, -1.0 when it saw no
// finite value) and the completion ticket.  Host code must not use this
// name as an address: it is a host-side stand-in; the device address comes
// from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned long long g_noalloc_scratch[kScratchWords];

struct DtArgs {
  const double *q;  // interleaved interior primitives, Ny x Nx x 4
  double *out;      // {dt, inv_dt_hyp, inv_dt_tc, inv_dt_visc}
  unsigned long long *scratch;
  long long ncells;
  int nblocks;
  double gamma, gm1, dx, dy, inv_dx, inv_dy;
  int dx_pow2, dy_pow2;
  uint64_t rw_dx, rw_dy;  // reciprocal words of dx, dy (quotients when 1/dx is inexact)
  double CFL, inv_tc, inv_visc;
};

__device__ __forceinline__ double div_spacing(double x, double d, double inv_d, int pow2, uint64_t rw) {
  return pow2 ? x * inv_d : fv2d::fv_div_by(x, d, rw);
}

// Same per-cell expression and the same max semantics as the dt reduction of
// the set-up pass and of the fused step (ComputeDt.h:31-34, 46-48), so the
// result is bit-identical to fv2d_compute_dt on the same state.
__global__ void __launch_bounds__(kThreads) dt_noalloc_kernel(DtArgs a) {
  __shared__ double red[kThreads / 32];
  __shared__ int s_last;
  const fv2d::Gas<double> gas = fv2d::make_gas(a.gamma, a.gm1, 1.0 / a.gm1, 0.0);
  double m = -1.0;
  const long long base = (long long)blockIdx.x * kCellsPerBlock;
#pragma unroll
  for (int k = 0; k < kCellsPerThread; ++k) {
    const long long c = base + (long long)k * kThreads + threadIdx.x;
    if (c < a.ncells) {
      const double *s = a.q + c * 4;
      const fv2d::S4<double> q{s[0], s[1], s[2], s[3]};
      const double cs = fv2d::sound_speed(q, gas);
      const double ih = div_spacing(cs + fabs(q.u), a.dx, a.inv_dx, a.dx_pow2, a.rw_dx) +
                        div_spacing(cs + fabs(q.v), a.dy, a.inv_dy, a.dy_pow2, a.rw_dy);
      m = fmax(m, ih);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    double b = -1.0;
    for (int w = 0; w < kThreads / 32; ++w) b = fmax(b, red[w]);
    a.scratch[blockIdx.x] = (unsigned long long)__double_as_longlong(b);
    __threadfence();
    const unsigned t = atomicAdd(reinterpret_cast<unsigned int *>(&a.scratch[kTicketSlot]), 1u);
    s_last = (t == (unsigned)a.nblocks - 1u);
  }
  __syncthreads();
  if (!s_last) return;
  // last CTA: reduce the partials, finish computeDt (ComputeDt.h:64)
  __threadfence();
  double r = -1.0;
  for (int b = threadIdx.x; b < a.nblocks; b += kThreads) {
    const volatile unsigned long long *p = a.scratch;
    r = fmax(r, __longlong_as_double((long long)p[b]));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) r = fmax(r, __shfl_xor_sync(0xffffffffu, r, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = r;
  __syncthreads();
  if (threadIdx.x == 0) {
    double hyp = -1.0;
    for (int w = 0; w < kThreads / 32; ++w) hyp = fmax(hyp, red[w]);
    if (!(hyp >= 0.0)) hyp = 0.0;
    double mx = hyp;
    if (mx < a.inv_tc) mx = a.inv_tc;
    if (mx < a.inv_visc) mx = a.inv_visc;
    a.out[0] = a.CFL / mx;
    a.out[1] = hyp;
    a.out[2] = a.inv_tc;
    a.out[3] = a.inv_visc;
    a.scratch[kTicketSlot] = 0ull;
  }
}

// Device address of the scratch array, looked up once per device and kept
// for the life of the process.  A device reset (cudaDeviceReset) or a new
// primary context reloads the module at another address, so the entry point
// must not be used on a device after it has been reset.
std::mutex g_mu;
void *g_scratch_addr[256];

bool pow2_spacing(double d) {
  if (!(d > 0) || !std::isfinite(d)) return false;
  int e;
  return std::frexp(d, &e) == 0.5 && std::isfinite(1.0 / d);
}

}  // namespace

extern "C" int fv2d_compute_dt_noalloc(const fv2d_params *p, const double *q_dev, double *out_dev, void *stream) {
  if (!p || !q_dev || !out_dev) return FV2D_ERR_INVALID;
  if (fv2d::validate(*p)) return FV2D_ERR_INVALID;
  const long long ncells = (long long)p->Nx * p->Ny;
  if (ncells > FV2D_NOALLOC_MAX_CELLS) return FV2D_ERR_SIZE;  // more partials than the fixed scratch holds
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 256) return FV2D_ERR_CUDA;
  void *scratch = nullptr;
  {
    // first call on this device: resolve the array's device address (with this
    // device current)
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_addr[dev]) {
      void *ptr = nullptr;
      if (cudaGetSymbolAddress(&ptr, g_noalloc_scratch) != cudaSuccess || !ptr) return FV2D_ERR_CUDA;
      g_scratch_addr[dev] = ptr;
    }
    scratch = g_scratch_addr[dev];
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // the completion ticket must start at zero
  if (cudaMemsetAsync(static_cast<unsigned long long *>(scratch) + kTicketSlot, 0, sizeof(unsigned long long), s) !=
      cudaSuccess)
    return FV2D_ERR_CUDA;
  DtArgs a;
  a.q = q_dev;
  a.out = out_dev;
  a.scratch = static_cast<unsigned long long *>(scratch);
  a.ncells = ncells;
  a.nblocks = (int)((ncells + kCellsPerBlock - 1) / kCellsPerBlock);
  a.gamma = p->gamma0;
  a.gm1 = p->gamma0 - 1.0;
  a.dx = (p->xmax - p->xmin) / p->Nx;
  a.dy = (p->ymax - p->ymin) / p->Ny;
  a.dx_pow2 = pow2_spacing(a.dx);
  a.dy_pow2 = pow2_spacing(a.dy);
  a.inv_dx = a.dx_pow2 ? 1.0 / a.dx : 0.0;
  a.inv_dy = a.dy_pow2 ? 1.0 / a.dy : 0.0;
  a.rw_dx = fv2d::softfp::recip_of_host(a.dx);
  a.rw_dy = fv2d::softfp::recip_of_host(a.dy);
  a.CFL = p->CFL;
  fv2d::parabolic_inv_dt(*p, &a.inv_tc, &a.inv_visc);
  dt_noalloc_kernel<<<a.nblocks, kThreads, 0, s>>>(a);
  return cudaGetLastError() == cudaSuccess ? FV2D_OK : FV2D_ERR_CUDA;
}
