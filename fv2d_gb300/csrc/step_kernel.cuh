// step_kernel.cuh -- the fused FP64 hydro step for sm_103a.
//
// One CTA owns a TX x TY tile of interior cells.  Per launch it
//   1. stages the tile plus its 2-cell halo of all four primitive planes
//      into shared memory with one 3-D TMA load (cp.async.bulk.tensor);
//   2. computes minmod slopes (Update.h:59-91) and, with thermal conduction,
//      the temperatures p/rho (ThermalConduction.h:56-60), once per cell;
//   3. solves every x- and y-face Riemann problem once (the reference solves
//      each twice, once from each neighbour: Update.h:142-143; both solves see
//      identical inputs, so the flux is the same);
//   4. accumulates the conservative update of each cell in the reference's
//      order -- x flux divergence, x gravity, y flux divergence, y gravity,
//      thermal conduction, viscosity (Update.h:158-172, 186-190,
//      ThermalConduction.h:106, Viscosity.h:112-117) -- and, for the RK2
//      corrector, the average with U0 (Update.h:214-220);
//   5. writes U once, converts to primitives and applies the
//      negative-density/pressure reset with its counters (SimInfo.h:576-636),
//      writes the primitive state into the other buffer including every ghost
//      cell that copies it (BoundaryConditions.h:82-147, inverse map), and
//      folds the next step's inverse hyperbolic dt (ComputeDt.h:26-52) into a
//      warp-shuffle max and one atomic per CTA;
//   6. a one-thread kernel that follows in stream order commits t += dt, the
//      counters and the next dt, and evaluates the device-driven loop
//      condition (main.cpp:62-64); the step's CTAs only fire their reduction
//      atomics and exit (no fence, no last-CTA election).
// Built with -fmad=false the results are bit-identical to the reference's
// binary64 arithmetic.
#pragma once

#include "physics.cuh"
#include "step_common.cuh"

namespace fv2d {

// ------------------------------------------------------------------ PTX helpers
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t phase) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(phase)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *tm, int x, int y, int z, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(tm)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

// Bounded wait on phase 0 of a one-shot barrier.  Gives up after ~seconds,
// records the error and waits (again bounded) so that no copy is left in
// flight into shared memory when the CTA exits.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, int *err_flag, uint32_t limit = 1u << 24) {
  for (uint32_t it = 0; it < limit; ++it)
    if (mbar_try_wait(bar, 0)) return true;
  atomicOr(err_flag, DEVERR_TMA_TIMEOUT);
  for (uint32_t it = 0; it < limit; ++it)
    if (mbar_try_wait(bar, 0)) break;
  return false;
}

__device__ __forceinline__ double ddivc(double x, double d, double inv_d, int pow2, uint64_t rw) {
  // x / d; when 1/d is exactly representable the product is the same
  // correctly rounded value; otherwise the quotient uses d's reciprocal word
  // rw, formed once on the host.
  if (pow2) return softfp::mul_pow2(x, inv_d, (int)((softfp::bits(inv_d) >> 52) & 0x7FF) - 1023);
  return fv_div_by(x, d, rw);
}

__device__ __forceinline__ double warp_max_nonneg(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ unsigned warp_sum(unsigned v) { return __reduce_add_sync(0xffffffffu, v); }

// Bounds-check build (-DFV2D_BOUNDS_CHECK, built for the tests as a stand-in
// for a memory checker): every shared-memory index and every global plane
// index of the step is checked; a bad one sets DEVERR_BOUNDS in the device
// state and is redirected to a scratch slot (shared memory) or skipped
// (global memory).  Without the macro the checks compile away.
#ifdef FV2D_BOUNDS_CHECK
constexpr bool kBoundsCheck = true;
#else
constexpr bool kBoundsCheck = false;
#endif
__device__ __forceinline__ int smem_index(int i, int total, int *err) {
  if (kBoundsCheck && (i < 0 || i >= total)) {
    atomicOr(err, DEVERR_BOUNDS);
    return total;  // the spare slot past the layout
  }
  return i;
}
__device__ __forceinline__ bool gidx_ok(long long i, long long n, int *err) {
  if (kBoundsCheck && (i < 0 || i >= n)) {
    atomicOr(err, DEVERR_BOUNDS);
    return false;
  }
  return true;
}

// Shared-memory layout (in doubles) for a reconstruction type, with or
// without the viscous face terms.
template <int RECON, bool VISC = false>
struct Smem {
  static constexpr int R1W = TX + 2, R1H = TY + 2;  // tile + 1-cell ring
  static constexpr int R1 = R1W * R1H;
  static constexpr int Q = 0;
  static constexpr int SX = Q + 4 * SH * SW;
  static constexpr int SY = SX + ((RECON != RECON_PCM) ? 4 * R1 : 0);
  static constexpr int QH = SY + ((RECON != RECON_PCM) ? 4 * R1 : 0);
  static constexpr int FX = QH + ((RECON == RECON_MH) ? 4 * R1 : 0);
  static constexpr int FY = FX + 4 * TY * (TX + 1);
  static constexpr int PY = FY + 4 * (TY + 1) * TX;
  static constexpr int T = PY + (TY + 1) * TX;
  static constexpr int VX = T + R1;                                  // viscous x-face terms, 3 x TY x (TX+1)
  static constexpr int VY = VX + (VISC ? 3 * TY * (TX + 1) : 0);     // viscous y-face terms, 3 x (TY+1) x TX
  static constexpr int TOTAL = VY + (VISC ? 3 * (TY + 1) * TX : 0);
  static constexpr size_t BYTES = sizeof(double) * (TOTAL + 1) + 128;  // + spare slot + alignment slack
};

// CTAs per SM: 3.  Without viscosity, measured faster with more at the price
// of register spills (their shared memory still fits): PCM with HLL or HLLC
// at 5 (40 registers), PCM with FSLP and PLM with HLL or FSLP at 4 (56); PLM
// and MUSCL-Hancock with HLLC stay at 3.
template <int RECON, int RS>
constexpr int step_ctas_per_sm(bool visc) {
  if (visc) return 3;
  if (RECON == RECON_PCM) return RS == RS_FSLP ? 4 : 5;
  if (RECON == RECON_PLM && RS != RS_HLLC) return 4;
  return 3;
}

template <int RECON, int RS, bool VISC>
__global__ void __launch_bounds__(NT, step_ctas_per_sm<RECON, RS>(VISC))
    step_kernel(const __grid_constant__ CUtensorMap tmQ0, const __grid_constant__ CUtensorMap tmQ1,
                const StepArgs a) {
  using L = Smem<RECON, VISC>;
  // Aligned by offsetting the shared array itself (not through an integer
  // round trip, which would turn every tile access into a generic load).
  extern __shared__ __align__(128) unsigned char fv2d_step_smem[];
  double *sm = reinterpret_cast<double *>(fv2d_step_smem + ((128u - ((uint32_t)__cvta_generic_to_shared(fv2d_step_smem) & 127u)) & 127u));
  __shared__ __align__(8) uint64_t mbar;
  __shared__ double red_max[NT / 32];
  __shared__ double s_tc[2];  // dt/dx, dt/dy of the conduction update (ThermalConduction.h:106), once per CTA
  __shared__ unsigned red_cnt[3][NT / 32];

  DevState *st = a.st;
  const int tid = threadIdx.x;
  if (a.driven && *((volatile int *)&st->status) != RUN_RUNNING) return;
  const int par = *((volatile int *)&st->parity);
  const double dt = a.driven ? *((volatile double *)&st->dt) : a.dt_arg;
  const int src = (a.stage == STAGE_RK2_CORRECT) ? 1 - par : par;
  const int dst = 1 - src;
  const CUtensorMap *tm = src ? &tmQ1 : &tmQ0;

  const int bx = blockIdx.x, by = blockIdx.y;
  const int i0 = bx * TX, j0 = by * TY;  // first interior cell of the tile

  // ---- 1. stage tile + halo (padded coordinates start at the halo) -------
  if (tid == 0) {
    mbar_init(&mbar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (tid == 0) {
    mbar_expect_tx(&mbar, 4u * SH * SW * sizeof(double));
    tma_load_3d(sm + L::Q, tm, i0, j0, 0, &mbar);
  }
  mbar_wait_bounded(&mbar, &st->error);

  auto SMI = [&](int i) -> double & { return sm[smem_index(i, L::TOTAL, &st->error)]; };
  auto gok = [&](long long i, long long n) { return gidx_ok(i, n, &st->error); };
  auto sQ = [&](int k, int ly, int lx) -> double & { return SMI(L::Q + (k * SH + ly) * SW + lx); };
  auto sR1 = [&](int base, int k, int ly, int lx) -> double & {
    return SMI(base + (k * L::R1H + (ly - 1)) * L::R1W + (lx - 1));
  };
  auto cellQ = [&](int ly, int lx) -> S4<double> {
    return S4<double>{sQ(0, ly, lx), sQ(1, ly, lx), sQ(2, ly, lx), sQ(3, ly, lx)};
  };
  const Gas<double> gas = make_gas(a.gamma, a.gm1, a.entho, a.fslp_K);

  // ---- 2. slopes (+ MUSCL-Hancock predictor) and temperatures ------------
  if constexpr (RECON == RECON_PLM) {
    // Neighbour differences, once per face (the dR of one cell is the dL of
    // the next: Update.h:70-76 computes both), held in the face-flux area
    // until the Riemann pass: DX[k][r][f] = Q(f+1) - Q(f) on padded row r+2,
    // DY[k][g][c] = Q(g+1) - Q(g) on padded column c+2.
    constexpr int NDX = 4 * TY * (TX + 3), NDY = 4 * (TY + 3) * TX;
    static_assert(NDX + NDY <= L::T - L::FX, "difference arrays exceed the face-flux area");
    // DX at L::FX, DY at L::FX + NDX
    for (int it = tid; it < NDX + NDY; it += NT) {
      if (it < NDX) {
        const int k = it / (TY * (TX + 3)), rem = it % (TY * (TX + 3));
        const int ly = rem / (TX + 3) + 2, lx = rem % (TX + 3) + 1;
        SMI(L::FX + it) = sQ(k, ly, lx) - sQ(k, ly, lx - 1);
      } else {
        const int jt = it - NDX;
        const int k = jt / ((TY + 3) * TX), rem = jt % ((TY + 3) * TX);
        const int ly = rem / TX + 1, lx = rem % TX + 2;
        SMI(L::FX + NDX + jt) = sQ(k, ly, lx) - sQ(k, ly - 1, lx);
      }
    }
    __syncthreads();
    // half slopes 0.5*minmod: x at rows [2,TY+2) x cols [1,TX+3),
    // y at rows [1,TY+3) x cols [2,TX+2)
    constexpr int NXS = TY * (TX + 2), NYS = (TY + 2) * TX;
    for (int it = tid; it < NXS + NYS; it += NT) {
      if (it < NXS) {
        const int r = it / (TX + 2), c = it % (TX + 2);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const int d = L::FX + (k * TY + r) * (TX + 3) + c;  // dL, dR of column c+1
          sR1(L::SX, k, r + 2, c + 1) = fv_half(minmod(SMI(d), SMI(d + 1)));
        }
      } else {
        const int jt = it - NXS;
        const int g = jt / TX, c = jt % TX;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const int d = L::FX + NDX + (k * (TY + 3) + g) * TX + c;  // dU, dD of row g+1
          sR1(L::SY, k, g + 1, c + 2) = fv_half(minmod(SMI(d), SMI(d + TX)));
        }
      }
    }
  } else if constexpr (RECON == RECON_MH) {
    for (int it = tid; it < L::R1; it += NT) {
      const int ly = it / L::R1W + 1, lx = it % L::R1W + 1;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const double c = sQ(k, ly, lx);
        sR1(L::SX, k, ly, lx) = minmod(c - sQ(k, ly, lx - 1), sQ(k, ly, lx + 1) - c);
        sR1(L::SY, k, ly, lx) = minmod(c - sQ(k, ly - 1, lx), sQ(k, ly + 1, lx) - c);
      }
    }
  }
  if (a.tc) {
    for (int it = tid; it < L::R1; it += NT) {
      const int ly = it / L::R1W + 1, lx = it % L::R1W + 1;
      sR1(L::T, 0, ly, lx) = fv_div(sQ(3, ly, lx), sQ(0, ly, lx));
    }
    if (tid == NT - 1) {
      s_tc[0] = fv_div(dt, a.dx);
      s_tc[1] = fv_div(dt, a.dy);
    }
  }
  __syncthreads();
  if constexpr (RECON == RECON_MH) {
    const double ax = fv_div(0.5 * dt, a.dx), ay = fv_div(0.5 * dt, a.dy);
    for (int it = tid; it < L::R1; it += NT) {
      const int ly = it / L::R1W + 1, lx = it % L::R1W + 1;
      S4<double> sx{sR1(L::SX, 0, ly, lx), sR1(L::SX, 1, ly, lx), sR1(L::SX, 2, ly, lx), sR1(L::SX, 3, ly, lx)};
      S4<double> sy{sR1(L::SY, 0, ly, lx), sR1(L::SY, 1, ly, lx), sR1(L::SY, 2, ly, lx), sR1(L::SY, 3, ly, lx)};
      S4<double> h = hancock(cellQ(ly, lx), sx, sy, ax, ay, a.gamma);
      sR1(L::QH, 0, ly, lx) = h.r;
      sR1(L::QH, 1, ly, lx) = h.u;
      sR1(L::QH, 2, ly, lx) = h.v;
      sR1(L::QH, 3, ly, lx) = h.p;
    }
    __syncthreads();
  }

  // Face state of cell (ly, lx) on side `plus` (+1 side if true) along dir.
  auto face_state = [&](int ly, int lx, bool plus, int dir) -> S4<double> {
    if constexpr (RECON == RECON_PCM) {
      return cellQ(ly, lx);
    } else if constexpr (RECON == RECON_PLM) {
      const int base = dir ? L::SY : L::SX;
      S4<double> q = cellQ(ly, lx);
      const double h0 = sR1(base, 0, ly, lx), h1 = sR1(base, 1, ly, lx), h2 = sR1(base, 2, ly, lx),
                   h3 = sR1(base, 3, ly, lx);
      // q + slope*sign*0.5 (Update.h:25) with the half slope precomputed
      if (plus) return S4<double>{q.r + h0, q.u + h1, q.v + h2, q.p + h3};
      return S4<double>{q.r + (-h0), q.u + (-h1), q.v + (-h2), q.p + (-h3)};
    } else {
      const int base = dir ? L::SY : L::SX;
      const double sg = plus ? 1.0 : -1.0;
      S4<double> q{sR1(L::QH, 0, ly, lx), sR1(L::QH, 1, ly, lx), sR1(L::QH, 2, ly, lx), sR1(L::QH, 3, ly, lx)};
      return S4<double>{q.r + sR1(base, 0, ly, lx) * sg * 0.5, q.u + sR1(base, 1, ly, lx) * sg * 0.5,
                        q.v + sR1(base, 2, ly, lx) * sg * 0.5, q.p + sR1(base, 3, ly, lx) * sg * 0.5};
    }
  };

  // ---- 3. face fluxes: x faces then y faces, one Riemann solve each ---------
  {
    constexpr int NFX = TY * (TX + 1), NFY = (TY + 1) * TX;
    for (int f = tid; f < NFX + NFY; f += NT) {
      const bool ydir = f >= NFX;
      int r, c, lyR, lxR, lyL, lxL;
      if (!ydir) {
        r = f / (TX + 1);
        c = f % (TX + 1);
        lyR = r + 2; lxR = c + 2; lyL = lyR; lxL = lxR - 1;
      } else {
        const int g = f - NFX;
        r = g / TX;
        c = g % TX;
        lyR = r + 2; lxR = c + 2; lyL = lyR - 1; lxL = lxR;
      }
      S4<double> qL = face_state(lyL, lxL, true, ydir);
      S4<double> qR = face_state(lyR, lxR, false, ydir);
      if (ydir) {  // swap_component (States.h:103-110)
        double t0 = qL.u; qL.u = qL.v; qL.v = t0;
        double t1 = qR.u; qR.u = qR.v; qR.v = t1;
      }
      S4<double> fl;
      double pout;
      riemann<RS>(qL, qR, fl, pout, ydir ? a.gy_dy : a.gx_dx, gas);
      if (!ydir) {
        const int F = L::FX + r * (TX + 1) + c;
        SMI(F) = fl.r;
        SMI(F + 1 * TY * (TX + 1)) = fl.u;
        SMI(F + 2 * TY * (TX + 1)) = fl.v;
        SMI(F + 3 * TY * (TX + 1)) = fl.p;
      } else {
        const int F = L::FY + r * TX + c;
        SMI(F) = fl.r;
        SMI(F + 1 * (TY + 1) * TX) = fl.v;  // swap back (Update.h:145-146)
        SMI(F + 2 * (TY + 1) * TX) = fl.u;
        SMI(F + 3 * (TY + 1) * TX) = fl.p;
        SMI(L::PY + r * TX + c) = pout;
      }
    }
  }
  // viscous face terms (Viscosity.h:63-107), once per face: the two cells of
  // a face evaluate the same expressions in the reference, the one on the
  // +side of the face with sign -1, which only negates the products exactly
  if constexpr (VISC) {
    constexpr double four_thirds = 4.0 / 3.0;
    constexpr double two_thirds = 2.0 / 3.0;
    const double mu = a.mu;
    const double odx = a.one_over_dx, ody = a.one_over_dy;
    const double q_odx = 0.25 * odx, q_ody = 0.25 * ody;  // (0.25 * ody) * (...) as the reference groups it
    constexpr int NVX = TY * (TX + 1), NVY = (TY + 1) * TX;
    for (int f = tid; f < NVX + NVY; f += NT) {
      if (f < NVX) {  // between columns c+1 (s-1) and c+2 (s) of row r+2
        const int r = f / (TX + 1), c = f % (TX + 1);
        const int ly = r + 2, xs = c + 2, xm = c + 1;
        auto U_ = [&](int dj, int x) { return sQ(1, ly + dj, x); };
        auto V_ = [&](int dj, int x) { return sQ(2, ly + dj, x); };
        const double qiu = fv_half(U_(0, xs) + U_(0, xm));
        const double qiv = fv_half(V_(0, xs) + V_(0, xm));
        const double dudx = mulx<11>(odx, U_(0, xs) - U_(0, xm));
        const double dvdx = mulx<11>(odx, V_(0, xs) - V_(0, xm));
        const double dudy = mulx<11>(q_ody, U_(1, xs) - U_(-1, xs) + U_(1, xm) - U_(-1, xm));
        const double dvdy = mulx<11>(q_ody, V_(1, xs) - V_(-1, xs) + V_(1, xm) - V_(-1, xm));
        const double tau_xx = mulx<11>(four_thirds, dudx) - mulx<11>(two_thirds, dvdy);
        const double tau_xy = dvdx + dudy;
        SMI(L::VX + f) = mulx<11>(mu, tau_xx);
        SMI(L::VX + f + NVX) = mulx<11>(mu, tau_xy);
        SMI(L::VX + f + 2 * NVX) = mulx<11>(mu, mulx<11>(tau_xx, qiu) + mulx<11>(tau_xy, qiv));
      } else {  // between rows r+1 (s-1) and r+2 (s) of column c+2
        const int g = f - NVX;
        const int r = g / TX, c = g % TX;
        const int lx = c + 2, ys = r + 2, ym = r + 1;
        auto U_ = [&](int y, int di) { return sQ(1, y, lx + di); };
        auto V_ = [&](int y, int di) { return sQ(2, y, lx + di); };
        const double qiu = fv_half(U_(ys, 0) + U_(ym, 0));
        const double qiv = fv_half(V_(ys, 0) + V_(ym, 0));
        const double dudy = mulx<11>(ody, U_(ys, 0) - U_(ym, 0));
        const double dvdy = mulx<11>(ody, V_(ys, 0) - V_(ym, 0));
        const double dudx = mulx<11>(q_odx, U_(ys, 1) - U_(ys, -1) + U_(ym, 1) - U_(ym, -1));
        const double dvdx = mulx<11>(q_odx, V_(ys, 1) - V_(ys, -1) + V_(ym, 1) - V_(ym, -1));
        const double tau_yy = mulx<11>(four_thirds, dvdy) - mulx<11>(two_thirds, dudx);
        const double tau_xy = dvdx + dudy;
        SMI(L::VY + g) = mulx<11>(mu, tau_xy);
        SMI(L::VY + g + NVY) = mulx<11>(mu, tau_yy);
        SMI(L::VY + g + 2 * NVY) = mulx<11>(mu, mulx<11>(tau_xy, qiu) + mulx<11>(tau_yy, qiv));
      }
    }
  }
  __syncthreads();

  // ---- 4./5. cell update, conversion, stores, reductions -------------------
  double lmax = -1.0;
  unsigned cnt_rho = 0, cnt_prs = 0, cnt_nan = 0;
  const bool final_stage = (a.stage != STAGE_RK2_PREDICT);
  const double *Usrc = (a.stage == STAGE_RK2_CORRECT) ? a.U1 : a.U;
  double *Udst = (a.stage == STAGE_RK2_PREDICT) ? a.U1 : a.U;
  double *Qd = a.Q[dst];
  const long long PL = a.plane;
  const int P = a.pitch;

#pragma unroll 1
  for (int cidx = tid; cidx < TX * TY; cidx += NT) {
    const int ry = cidx / TX, rx = cidx % TX;
    const int i = i0 + rx, j = j0 + ry;
    if (i >= a.Nx || j >= a.Ny) continue;
    const int ly = ry + 2, lx = rx + 2;
    const long long g = (long long)(j + HALO) * P + (i + HALO);
    if (!gok(g, PL)) continue;
    double un[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) un[k] = Usrc[k * PL + g];
    const double rho = sQ(0, ly, lx);

    // x direction (Update.h:114-168 with dir = IX)
    {
      const int F = L::FX + ry * (TX + 1) + rx;
      constexpr int S = TY * (TX + 1);
      const double FL0 = SMI(F), FR0 = SMI(F + 1);
#pragma unroll
      for (int k = 0; k < 4; ++k)
        un[k] += ddivc(mulx<3>(SMI(F + k * S) - SMI(F + k * S + 1), dt), a.dx, a.inv_dx, a.dx_pow2, a.rw_dx);
      if (a.grav_mode) {
        const double gv = (a.grav_mode == 1) ? a.gxf : (double)a.grav_row[j];
        un[2] += dt * rho * gv;
        un[3] += dt * 0.5 * (FL0 + FR0) * gv;
      }
    }
    // y direction (dir = IY), with the well-balanced boundary override
    {
      const int F = L::FY + ry * TX + rx;
      constexpr int S = (TY + 1) * TX;
      double FL[4], FR[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        FL[k] = SMI(F + k * S);
        FR[k] = SMI(F + k * S + TX);
      }
      double gv = 0.0;
      if (a.grav_mode) gv = (a.grav_mode == 1) ? a.gyf : (double)a.grav_row[j];
      if (a.wb && (j == 0 || j == a.Ny - 1)) {  // Update.h:149-156
        const double gy = (a.grav_mode == 0) ? 0.0 : gv;
        if (j == 0) {
          const double poutR = SMI(L::PY + (ry + 1) * TX + rx);
          FL[0] = 0.0; FL[1] = 0.0; FL[2] = poutR - rho * gy * a.dy; FL[3] = 0.0;
        } else {
          const double poutL = SMI(L::PY + ry * TX + rx);
          FR[0] = 0.0; FR[1] = 0.0; FR[2] = poutL + rho * gy * a.dy; FR[3] = 0.0;
        }
      }
#pragma unroll
      for (int k = 0; k < 4; ++k) un[k] += ddivc(mulx<3>(FL[k] - FR[k], dt), a.dy, a.inv_dy, a.dy_pow2, a.rw_dy);
      if (a.grav_mode) {
        un[2] += dt * rho * gv;
        un[3] += dt * 0.5 * (FL[0] + FR[0]) * gv;
      }
    }
    // thermal conduction (ThermalConduction.h:46-106)
    if (a.tc) {
      const double TC = sR1(L::T, 0, ly, lx);
      const double TL = sR1(L::T, 0, ly, lx - 1), TR = sR1(L::T, 0, ly, lx + 1);
      const double TU = sR1(L::T, 0, ly - 1, lx), TD = sR1(L::T, 0, ly + 1, lx);
      const double kL = a.kap_row[4 * j + 0], kR = a.kap_row[4 * j + 1];
      const double kU = a.kap_row[4 * j + 2], kD = a.kap_row[4 * j + 3];
      double FLt = ddivc(mulx<12>(kL, TC - TL), a.dx, a.inv_dx, a.dx_pow2, a.rw_dx);
      double FRt = ddivc(mulx<12>(kR, TR - TC), a.dx, a.inv_dx, a.dx_pow2, a.rw_dx);
      const double FUt = ddivc(mulx<12>(kU, TC - TU), a.dy, a.inv_dy, a.dy_pow2, a.rw_dy);
      const double FDt = ddivc(mulx<12>(kD, TD - TC), a.dy, a.inv_dy, a.dy_pow2, a.rw_dy);
      if (j == 0 && a.bctc_ymin != 0) {
        if (a.bctc_ymin == 1)
          FLt = ddivc(kL * 2.0 * (TC - a.bctc_ymin_value), a.dy, a.inv_dy, a.dy_pow2, a.rw_dy);
        else
          FLt = kL * a.bctc_ymin_value;
      }
      if (j == a.Ny - 1 && a.bctc_ymax != 0) {
        if (a.bctc_ymax == 1)
          FRt = ddivc(kR * 2.0 * (a.bctc_ymax_value - TC), a.dy, a.inv_dy, a.dy_pow2, a.rw_dy);
        else
          FRt = kR * a.bctc_ymax_value;
      }
      un[3] += mulx<12>(s_tc[0], FRt - FLt) + mulx<12>(s_tc[1], FDt - FUt);
    }
    // viscosity (Viscosity.h:63-107): the face terms of the face pass, the
    // -side face negated, accumulated in the reference's order
    if constexpr (VISC) {
      constexpr int NVX = TY * (TX + 1), NVY = (TY + 1) * TX;
      const int Vw = L::VX + ry * (TX + 1) + rx;  // x face at rx (west), rx + 1 (east)
      const int Vn = L::VY + ry * TX + rx;        // y face at ry (north), ry + 1 (south)
      double fx1 = 0.0, fx2 = 0.0, fx3 = 0.0, fy1 = 0.0, fy2 = 0.0, fy3 = 0.0;
      fx1 += -SMI(Vw);
      fx2 += -SMI(Vw + NVX);
      fx3 += -SMI(Vw + 2 * NVX);
      fy1 += -SMI(Vn);
      fy2 += -SMI(Vn + NVY);
      fy3 += -SMI(Vn + 2 * NVY);
      fx1 += SMI(Vw + 1);
      fx2 += SMI(Vw + NVX + 1);
      fx3 += SMI(Vw + 2 * NVX + 1);
      fy1 += SMI(Vn + TX);
      fy2 += SMI(Vn + NVY + TX);
      fy3 += SMI(Vn + 2 * NVY + TX);
      un[0] += (0.0 + 0.0) * dt;
      un[1] += mulx<12>(fx1 + fy1, dt);
      un[2] += mulx<12>(fx2 + fy2, dt);
      un[3] += mulx<12>(fx3 + fy3, dt);
    }
    // RK2 corrector: 0.5 * (U0 + Unew) (Update.h:214-220)
    if (a.stage == STAGE_RK2_CORRECT) {
#pragma unroll
      for (int k = 0; k < 4; ++k) un[k] = 0.5 * (a.U[k * PL + g] + un[k]);
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) Udst[k * PL + g] = un[k];

    // consToPrim (+ checkNegatives on the final stage)
    S4<double> q = cons_to_prim(S4<double>{un[0], un[1], un[2], un[3]}, gas);
    if (final_stage) {
      if (fv_lt0(q.r)) { q.r = a.eps_reset; ++cnt_rho; }
      if (fv_lt0(q.p)) { q.p = a.eps_reset; ++cnt_prs; }
      cnt_nan += (unsigned)fv_isnan(q.r) + (unsigned)fv_isnan(q.u) + (unsigned)fv_isnan(q.v) + (unsigned)fv_isnan(q.p);
      // inverse hyperbolic dt of the new state (ComputeDt.h:31-34)
      const double cs = sound_speed(q, gas);
      const double ih = ddivc(cs + fabs(q.u), a.dx, a.inv_dx, a.dx_pow2, a.rw_dx) +
                        ddivc(cs + fabs(q.v), a.dy, a.inv_dy, a.dy_pow2, a.rw_dy);
      lmax = fv_fmax(lmax, ih);
    }
    Qd[g] = q.r;
    Qd[PL + g] = q.u;
    Qd[2 * PL + g] = q.v;
    Qd[3 * PL + g] = q.p;
    if (final_stage && a.mirror && gok((long long)j * a.Nx + i, (long long)a.Nx * a.Ny)) {
      // interleaved interior copy in host memory (over the C2C link)
      double2 *m = reinterpret_cast<double2 *>(a.mirror + ((long long)j * a.Nx + i) * 4);
      m[0] = make_double2(q.r, q.u);
      m[1] = make_double2(q.v, q.p);
    }
    // ghost cells that copy this cell (BoundaryConditions.h:82-147)
    const bool ex = (i < 2 || i >= a.Nx - 2), ey = (j < 2 || j >= a.Ny - 2);
    if (ex || ey) {
      int tx[5], ty[5];
      bool nx[5], ny[5];
      tx[0] = i; nx[0] = false;
      ty[0] = j; ny[0] = false;
      const int cx = 1 + (ex ? ghost_targets(i, a.Nx, a.bcx, tx + 1, nx + 1) : 0);
      const int cy = 1 + (ey ? ghost_targets(j, a.Ny, a.bcy, ty + 1, ny + 1) : 0);
      for (int b = 0; b < cy; ++b)
        for (int c = 0; c < cx; ++c) {
          if (b == 0 && c == 0) continue;
          const long long gg = (long long)(ty[b] + HALO) * P + (tx[c] + HALO);
          if (!gok(gg, PL)) continue;
          Qd[gg] = q.r;
          Qd[PL + gg] = nx[c] ? q.u * -1.0 : q.u;
          Qd[2 * PL + gg] = ny[b] ? q.v * -1.0 : q.v;
          Qd[3 * PL + gg] = q.p;
        }
    }
  }

  if (!final_stage) return;

  // ---- block reductions, one atomic per CTA --------------------------------
  const int warp = tid >> 5, lane = tid & 31;
  lmax = warp_max_nonneg(lmax);
  const unsigned w0 = warp_sum(cnt_rho), w1 = warp_sum(cnt_prs), w2 = warp_sum(cnt_nan);
  if (lane == 0) {
    red_max[warp] = lmax;
    red_cnt[0][warp] = w0;
    red_cnt[1][warp] = w1;
    red_cnt[2][warp] = w2;
  }
  __syncthreads();
  if (tid == 0) {
    double m = -1.0;
    unsigned c0 = 0, c1 = 0, c2 = 0;
    for (int w = 0; w < NT / 32; ++w) {
      m = fmax(m, red_max[w]);
      c0 += red_cnt[0][w];
      c1 += red_cnt[1][w];
      c2 += red_cnt[2][w];
    }
    // reductions only (no value returned, no fence): the commit kernel that
    // follows in stream order reads the totals
    if (m >= 0.0) atomicMax(&st->acc_hyp, (unsigned long long)__double_as_longlong(m));
    if (c0) atomicAdd(&st->cnt_acc[0], (unsigned long long)c0);
    if (c1) atomicAdd(&st->cnt_acc[1], (unsigned long long)c1);
    if (c2) atomicAdd(&st->cnt_acc[2], (unsigned long long)c2);
  }
}

// ---- 6. commit the step (one thread, after the step kernel in stream order):
// t += dt, the counters, the next dt, the per-iteration log and the
// device-driven loop condition (main.cpp:62-64, 83; ComputeDt.h:64).
static __global__ void commit_kernel(const StepArgs a) {
  DevState *st = a.st;
  volatile DevState *vs = st;
  if (a.driven && vs->status != RUN_RUNNING) return;
  const int par = vs->parity;
  const double dt = a.driven ? vs->dt : a.dt_arg;
  const double inv_prev = vs->inv_hyp;
  const double t_before = vs->t;
  const double inv_hyp = __longlong_as_double((long long)vs->acc_hyp);
  double m = inv_hyp;  // std::max({hyp, tc, visc}) (ComputeDt.h:64)
  if (m < a.inv_tc) m = a.inv_tc;
  if (m < a.inv_visc) m = a.inv_visc;
  const double dt_next = a.CFL / m;
  const double t_after = t_before + dt;
  vs->t = t_after;
  vs->last_dt = dt;
  vs->inv_hyp = inv_hyp;
  vs->dt = dt_next;
  const int ite = vs->ite;
  vs->ite = ite + 1;
  if (a.stage == STAGE_EULER) vs->parity = 1 - par;
  unsigned long long cnt[3];
  for (int k = 0; k < 3; ++k) {
    cnt[k] = vs->cnt_acc[k];
    vs->counters[k] = cnt[k];
    st->cnt_acc[k] = 0ull;
  }
  st->acc_hyp = 0ull;
  const int n = vs->steps_in_call;
  if (a.log && n < vs->log_cap) {
    double *rec = a.log + 6 * n;
    rec[0] = t_before;
    rec[1] = dt;
    rec[2] = inv_prev;
    rec[3] = (double)cnt[0];
    rec[4] = (double)cnt[1];
    rec[5] = (double)cnt[2];
  }
  vs->steps_in_call = n + 1;
  if (a.driven) {
    int s = RUN_RUNNING;
    if (!(t_after + vs->eps < vs->tend))
      s = RUN_DONE;  // main.cpp:62
    else if (vs->check_save && t_after + vs->eps > vs->next_save)
      s = RUN_SAVE;  // main.cpp:64
    else if (!(dt_next > 0.0) || isnan(dt_next) || isinf(dt_next))
      s = RUN_NUMERIC;
    else if (n + 1 >= vs->max_steps)
      s = RUN_PAUSED;
    vs->status = s;
  }
}


}  // namespace fv2d
