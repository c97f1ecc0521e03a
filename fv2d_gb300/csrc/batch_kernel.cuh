// batch_kernel.cuh -- one FP32 step of every active simulation of a batch.
//
// Persistent CTAs walk a (simulation, tile) work list (tiles of different
// simulations of one grid-size bucket, interleaved).  Per tile:
//   - stage the conservative tile + 2-cell halo (ghost ring stored with the
//     state) into shared memory, by one TMA load from the simulation's tensor
//     map or by cooperative 16-byte loads (STAGING, picked by the autotuner);
//   - consToPrim with the negative reset (States.h:32-43, SimInfo.h:618-627);
//     low-Mach simulations recover p = (E - Ek)(gamma - 1) in binary64
//     where it cancels (pressure_of);
//   - minmod half slopes, one Riemann solve per face (HLL or HLLC), update
//     in the reference's order (x flux, x gravity, y flux, y gravity,
//     conduction, viscosity) in binary32 with fused multiply-adds;
//   - store the new state in the other buffer, ghost copies included, and
//     fold the inverse hyperbolic dt into one atomic max per tile;
//   - the last tile of a simulation commits its step: t += dt in binary64,
//     next dt = CFL / max(inv_hyp, inv_tc, inv_visc) in binary64, buffer
//     flip, stop test (step count or end time).
// Simulations never exchange data, so results do not depend on which other
// simulations share the launch.
#pragma once

#include "batch_common.cuh"
#include "physics.cuh"

namespace fv2d {

namespace bk {
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
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
}  // namespace bk

template <int TX, int TY>
struct BatchSmem {
  static constexpr int SW = TX + 4, SH = TY + 4;
  static constexpr int R1W = TX + 2, R1H = TY + 2, R1 = R1W * R1H;
  static constexpr int Q = 0;                       // 4 x SH x SW (U, then Q in place)
  static constexpr int HX = Q + 4 * SH * SW;        // 4 x R1 half slopes x
  static constexpr int HY = HX + 4 * R1;            // 4 x R1 half slopes y
  static constexpr int FX = HY + 4 * R1;            // 4 x TY x (TX+1)
  static constexpr int FY = FX + 4 * TY * (TX + 1); // 4 x (TY+1) x TX
  static constexpr int T = FY + 4 * (TY + 1) * TX;  // R1 temperatures
  static constexpr int TOTAL = T + R1;
  static constexpr size_t BYTES = sizeof(float) * TOTAL + 128;
};

template <int TX, int TY, int NT, int STAGING>
__global__ void __launch_bounds__(NT) batch_step_kernel(const BatchArgs a) {
  using L = BatchSmem<TX, TY>;
  constexpr int SW = L::SW, SH = L::SH;
  // Aligned by offsetting the shared array itself (not through an integer
  // round trip, which would turn every tile access into a generic load).
  extern __shared__ __align__(128) unsigned char fv2d_batch_smem[];
  float *sm = reinterpret_cast<float *>(fv2d_batch_smem + ((128u - ((uint32_t)__cvta_generic_to_shared(fv2d_batch_smem) & 127u)) & 127u));
  __shared__ SimDev S;
  __shared__ __align__(8) uint64_t mbar;
  __shared__ float red_max[NT / 32];
  __shared__ unsigned red_neg[NT / 32];
  __shared__ unsigned red_nan[NT / 32];
  __shared__ int s_last;
  const int tid = threadIdx.x;
  uint32_t phase = 0;
  if (STAGING == 1) {
    if (tid == 0) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bk::smem_u32(&mbar)) : "memory");
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
  }
  const int nw = *a.n_work;

  auto sQ = [&](int k, int ly, int lx) -> float & { return sm[L::Q + (k * SH + ly) * SW + lx]; };
  auto sR = [&](int base, int k, int ly, int lx) -> float & {
    return sm[base + (k * L::R1H + (ly - 1)) * L::R1W + (lx - 1)];
  };

  for (int w = blockIdx.x; w < nw; w += gridDim.x) {
    const WorkItem item = a.work[w];
    if (tid < (int)(sizeof(SimDev) / 4)) {
      reinterpret_cast<int *>(&S)[tid] = reinterpret_cast<const volatile int *>(&a.sims[item.sim])[tid];
    }
    __syncthreads();
    if (S.status != SIM_ACTIVE) {
      __syncthreads();
      continue;
    }
    const int Nx = S.Nx, Ny = S.Ny, P = S.pitch;
    const long long PL = S.plane;
    const int cur = S.cur;
    const StageBuffers B = stage_buffers(S.U, cur, S.ts, S.stage);
    const float *src = B.src;
    float *dst = B.dst;
    const int sbuf = (B.src == S.U[cur]) ? cur : 1 - cur;  // the buffer staged by TMA
    const int i0 = item.tx * TX, j0 = item.ty * TY;
    const float dt = (float)S.dt;
    const Gas<float> gas{S.gamma, S.gm1, S.entho, 1.1f};

    // ---- stage the conservative tile + halo -----------------------------
    if (STAGING == 1 && S.tma_ok) {
      if (tid == 0) {
        const CUtensorMap *tm = a.tmaps + 2 * item.sim + sbuf;
        asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(reinterpret_cast<uint64_t>(tm))
                     : "memory");
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bk::smem_u32(&mbar)),
                     "r"((uint32_t)(4 * SH * SW * sizeof(float)))
                     : "memory");
        asm volatile(
            "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
            "[%5];" ::"r"(bk::smem_u32(sm + L::Q)),
            "l"(reinterpret_cast<uint64_t>(tm)), "r"(i0), "r"(j0), "r"(0), "r"(bk::smem_u32(&mbar))
            : "memory");
      }
      // bounded wait; a copy that outlives it fails this simulation (its
      // commit reads dev_err) and is waited for once more, bounded, before
      // the tile buffer is used again; one that outlives that too stops the
      // CTA and raises the launch's fault flag, which stops the service
      bool ok = false;
      const uint32_t limit = *(volatile unsigned int *)(a.ctl + 1);
      for (uint32_t it = 0; it < limit && !ok; ++it) ok = bk::mbar_try_wait(&mbar, phase);
      if (__syncthreads_or(!ok)) {
        if (tid == 0) atomicOr(&a.sims[item.sim].dev_err, (unsigned)BATCH_ERR_TMA_TIMEOUT);
        for (uint32_t it = 0; it < kTileWaitFinal && !ok; ++it) ok = bk::mbar_try_wait(&mbar, phase);
        if (__syncthreads_or(!ok)) {
          if (tid == 0) atomicOr(a.ctl, (unsigned)BATCH_ERR_TMA_TIMEOUT);
          return;
        }
      }
      phase ^= 1u;
    } else {
      constexpr int PER = SH * SW;
      for (int e = tid; e < 4 * PER; e += NT) {
        const int k = e / PER, r = e % PER;
        const int ly = r / SW, lx = r % SW;
        const int gy = j0 + ly, gx = i0 + lx;  // padded coordinates
        float v = 0.f;
        if (gx < Nx + 4 && gy < Ny + 4) v = __ldg(src + k * PL + (long long)gy * P + gx);
        sm[L::Q + e] = v;
      }
    }
    __syncthreads();

    // ---- conservative offsets -> primitive in place, negative reset except
    //      in the second RK2 stage (whose Q is consToPrim(U*) alone) ---------
    for (int e = tid; e < SH * SW; e += NT) {
      const int ly = e / SW, lx = e % SW;
      float r = sQ(0, ly, lx) + S.bg_r, mu = sQ(1, ly, lx), mv = sQ(2, ly, lx), dE = sQ(3, ly, lx);
      float u = mu / r, v = mv / r;
      float p = pressure_of(dE, S.bg_e, r, u, v, S.gm1, S.lowmach);
      if (!B.avg) {
        if (r < 0.f) r = 1e-8f;
        if (p < 0.f) p = 1e-8f;
      }
      sQ(0, ly, lx) = r;
      sQ(1, ly, lx) = u;
      sQ(2, ly, lx) = v;
      sQ(3, ly, lx) = p;
    }
    __syncthreads();

    // ---- half slopes and temperatures --------------------------------------
    if (S.recon == 2) {
      constexpr int NXS = TY * (TX + 2), NYS = (TY + 2) * TX;
      for (int e = tid; e < NXS + NYS; e += NT) {
        if (e < NXS) {
          const int ly = e / (TX + 2) + 2, lx = e % (TX + 2) + 1;
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            const float c = sQ(k, ly, lx);
            sR(L::HX, k, ly, lx) = minmod(c - sQ(k, ly, lx - 1), sQ(k, ly, lx + 1) - c) * 0.5f;
          }
        } else {
          const int f = e - NXS;
          const int ly = f / TX + 1, lx = f % TX + 2;
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            const float c = sQ(k, ly, lx);
            sR(L::HY, k, ly, lx) = minmod(c - sQ(k, ly - 1, lx), sQ(k, ly + 1, lx) - c) * 0.5f;
          }
        }
      }
    }
    if (S.tc) {
      for (int e = tid; e < L::R1; e += NT) {
        const int ly = e / L::R1W + 1, lx = e % L::R1W + 1;
        sR(L::T, 0, ly, lx) = sQ(3, ly, lx) / sQ(0, ly, lx);
      }
    }
    __syncthreads();

    // ---- faces ---------------------------------------------------------------
    {
      constexpr int NFX = TY * (TX + 1), NFY = (TY + 1) * TX;
      const bool plm = S.recon == 2;
      const bool hll = S.rs == RS_HLL;
      for (int f = tid; f < NFX + NFY; f += NT) {
        const bool ydir = f >= NFX;
        int r, c, lyR, lxR, lyL, lxL;
        if (!ydir) {
          r = f / (TX + 1); c = f % (TX + 1);
          lyR = r + 2; lxR = c + 2; lyL = lyR; lxL = lxR - 1;
        } else {
          const int g = f - NFX;
          r = g / TX; c = g % TX;
          lyR = r + 2; lxR = c + 2; lyL = lyR - 1; lxL = lxR;
        }
        S4<float> qL{sQ(0, lyL, lxL), sQ(1, lyL, lxL), sQ(2, lyL, lxL), sQ(3, lyL, lxL)};
        S4<float> qR{sQ(0, lyR, lxR), sQ(1, lyR, lxR), sQ(2, lyR, lxR), sQ(3, lyR, lxR)};
        if (plm) {
          const int base = ydir ? L::HY : L::HX;
          qL.r += sR(base, 0, lyL, lxL); qL.u += sR(base, 1, lyL, lxL);
          qL.v += sR(base, 2, lyL, lxL); qL.p += sR(base, 3, lyL, lxL);
          qR.r -= sR(base, 0, lyR, lxR); qR.u -= sR(base, 1, lyR, lxR);
          qR.v -= sR(base, 2, lyR, lxR); qR.p -= sR(base, 3, lyR, lxR);
        }
        if (ydir) {
          float t0 = qL.u; qL.u = qL.v; qL.v = t0;
          float t1 = qR.u; qR.u = qR.v; qR.v = t1;
        }
        S4<float> fl;
        float pout;
        if (hll)
          riemann_hll(qL, qR, fl, pout, gas);
        else
          riemann_hllc(qL, qR, fl, pout, gas);
        if (!ydir) {
          float *F = sm + L::FX + r * (TX + 1) + c;
          F[0] = fl.r; F[TY * (TX + 1)] = fl.u; F[2 * TY * (TX + 1)] = fl.v; F[3 * TY * (TX + 1)] = fl.p;
        } else {
          float *F = sm + L::FY + r * TX + c;
          F[0] = fl.r; F[(TY + 1) * TX] = fl.v; F[2 * (TY + 1) * TX] = fl.u; F[3 * (TY + 1) * TX] = fl.p;
        }
      }
    }
    __syncthreads();

    // ---- update, store, reductions --------------------------------------------
    float lmax = 0.f;
    unsigned nneg = 0, nnan = 0;
    const float dtdx = dt * S.inv_dx, dtdy = dt * S.inv_dy;
    for (int cidx = tid; cidx < TX * TY; cidx += NT) {
      const int ry = cidx / TX, rx = cidx % TX;
      const int i = i0 + rx, j = j0 + ry;
      if (i >= Nx || j >= Ny) continue;
      const int ly = ry + 2, lx = rx + 2;
      const long long g = (long long)(j + 2) * P + (i + 2);
      float un[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) un[k] = src[k * PL + g];
      const float rho = sQ(0, ly, lx);
      {
        const float *F = sm + L::FX + ry * (TX + 1) + rx;
        constexpr int SX = TY * (TX + 1);
#pragma unroll
        for (int k = 0; k < 4; ++k) un[k] += (F[k * SX] - F[k * SX + 1]) * dtdx;
        if (S.grav) {
          un[2] += dt * rho * S.gx;
          un[3] += dt * 0.5f * (F[0] + F[1]) * S.gx;
        }
      }
      {
        const float *F = sm + L::FY + ry * TX + rx;
        constexpr int SY = (TY + 1) * TX;
#pragma unroll
        for (int k = 0; k < 4; ++k) un[k] += (F[k * SY] - F[k * SY + TX]) * dtdy;
        if (S.grav) {
          un[2] += dt * rho * S.gy;
          un[3] += dt * 0.5f * (F[0] + F[TX]) * S.gy;
        }
      }
      if (S.tc) {
        const float TC = sR(L::T, 0, ly, lx);
        const float FL = S.kappa * (TC - sR(L::T, 0, ly, lx - 1)) * S.inv_dx;
        const float FR = S.kappa * (sR(L::T, 0, ly, lx + 1) - TC) * S.inv_dx;
        const float FU = S.kappa * (TC - sR(L::T, 0, ly - 1, lx)) * S.inv_dy;
        const float FD = S.kappa * (sR(L::T, 0, ly + 1, lx) - TC) * S.inv_dy;
        un[3] += dtdx * (FR - FL) + dtdy * (FD - FU);
      }
      if (S.visc) {
        const float mu = S.mu, odx = S.inv_dx, ody = S.inv_dy;
        auto U_ = [&](int dj, int di) { return sQ(1, ly + dj, lx + di); };
        auto V_ = [&](int dj, int di) { return sQ(2, ly + dj, lx + di); };
        float f1 = 0.f, f2 = 0.f, f3 = 0.f;
#pragma unroll
        for (int side = 1; side < 3; ++side) {
          const float sign = side == 1 ? -1.f : 1.f;
          const int s = side - 1, sm1 = side - 2;
          {
            const float qiu = (U_(0, s) + U_(0, sm1)) * 0.5f, qiv = (V_(0, s) + V_(0, sm1)) * 0.5f;
            const float dudx = odx * (U_(0, s) - U_(0, sm1)), dvdx = odx * (V_(0, s) - V_(0, sm1));
            const float dudy = 0.25f * ody * (U_(1, s) - U_(-1, s) + U_(1, sm1) - U_(-1, sm1));
            const float dvdy = 0.25f * ody * (V_(1, s) - V_(-1, s) + V_(1, sm1) - V_(-1, sm1));
            const float txx = (4.f / 3.f) * dudx - (2.f / 3.f) * dvdy, txy = dvdx + dudy;
            f1 += sign * mu * txx; f2 += sign * mu * txy; f3 += sign * mu * (txx * qiu + txy * qiv);
          }
          {
            const float qiu = (U_(s, 0) + U_(sm1, 0)) * 0.5f, qiv = (V_(s, 0) + V_(sm1, 0)) * 0.5f;
            const float dudy = ody * (U_(s, 0) - U_(sm1, 0)), dvdy = ody * (V_(s, 0) - V_(sm1, 0));
            const float dudx = 0.25f * odx * (U_(s, 1) - U_(s, -1) + U_(sm1, 1) - U_(sm1, -1));
            const float dvdx = 0.25f * odx * (V_(s, 1) - V_(s, -1) + V_(sm1, 1) - V_(sm1, -1));
            const float tyy = (4.f / 3.f) * dvdy - (2.f / 3.f) * dudx, txy = dvdx + dudy;
            f1 += sign * mu * txy; f2 += sign * mu * tyy; f3 += sign * mu * (txy * qiu + tyy * qiv);
          }
        }
        un[1] += f1 * dt; un[2] += f2 * dt; un[3] += f3 * dt;
      }
      if (B.avg) {  // SSP-RK2: 0.5 (U^n + U**) (Update.h:214-220), offsets alike
#pragma unroll
        for (int k = 0; k < 4; ++k) un[k] = 0.5f * (dst[k * PL + g] + un[k]);
      }
#pragma unroll
      for (int k = 0; k < 4; ++k) dst[k * PL + g] = un[k];
      if (B.last) {
        // primitive state of the new cell for the next dt
        float r = un[0] + S.bg_r, u = un[1] / r, v = un[2] / r;
        float p = pressure_of(un[3], S.bg_e, r, u, v, S.gm1, S.lowmach);
        nnan += is_nan_f(r) | is_nan_f(u) | is_nan_f(v) | is_nan_f(p);
        nneg += (r < 0.f) + (p < 0.f);
        if (r < 0.f) r = 1e-8f;
        if (p < 0.f) p = 1e-8f;
        const float cs = sqrtf(p * S.gamma / r);
        const float ih = (cs + fabsf(u)) * S.inv_dx + (cs + fabsf(v)) * S.inv_dy;
        if (ih > lmax) lmax = ih;  // NaN never enters
      } else {
        nnan += is_nan_f(un[0]) | is_nan_f(un[1]) | is_nan_f(un[2]) | is_nan_f(un[3]);
      }
      // ghost copies (BoundaryConditions.h:82-147, inverse map)
      const bool ex = (i < 2 || i >= Nx - 2), ey = (j < 2 || j >= Ny - 2);
      if (ex || ey) {
        int tx[5], ty[5];
        bool nx[5], ny[5];
        tx[0] = i; nx[0] = false;
        ty[0] = j; ny[0] = false;
        const int cx = 1 + (ex ? ghost_targets(i, Nx, S.bcx, tx + 1, nx + 1) : 0);
        const int cy = 1 + (ey ? ghost_targets(j, Ny, S.bcy, ty + 1, ny + 1) : 0);
        for (int b = 0; b < cy; ++b)
          for (int c = 0; c < cx; ++c) {
            if (b == 0 && c == 0) continue;
            const long long gg = (long long)(ty[b] + 2) * P + (tx[c] + 2);
            dst[gg] = un[0];
            dst[PL + gg] = nx[c] ? -un[1] : un[1];
            dst[2 * PL + gg] = ny[b] ? -un[2] : un[2];
            dst[3 * PL + gg] = un[3];
          }
      }
    }
    // tile reductions
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) lmax = fmaxf(lmax, __shfl_xor_sync(0xffffffffu, lmax, o));
    const unsigned wn = __reduce_add_sync(0xffffffffu, nneg);
    const unsigned wnan = __reduce_add_sync(0xffffffffu, nnan);
    if ((tid & 31) == 0) {
      red_max[tid >> 5] = lmax;
      red_neg[tid >> 5] = wn;
      red_nan[tid >> 5] = wnan;
    }
    __syncthreads();
    if (tid == 0) {
      float m = 0.f;
      unsigned n = 0, nn = 0;
      for (int k = 0; k < NT / 32; ++k) {
        m = fmaxf(m, red_max[k]);
        n += red_neg[k];
        nn += red_nan[k];
      }
      SimDev *G = &a.sims[item.sim];
      if (B.last) atomicMax(&G->acc_bits, __float_as_uint(m));
      if (n) atomicAdd(&G->negatives, (unsigned long long)n);
      if (nn) atomicAdd(&G->nan_cells, nn);
      __threadfence();
      const unsigned t = atomicAdd(&G->ticket, 1u);
      s_last = (t == (unsigned)(S.ntx * S.nty) - 1u);
    }
    __syncthreads();
    if (s_last && tid == 0) commit_stage(&a.sims[item.sim]);  // ComputeDt.h:64, main.cpp:62, 83
    __syncthreads();
  }
}

}  // namespace fv2d
