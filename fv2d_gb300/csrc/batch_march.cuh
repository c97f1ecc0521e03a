// batch_march.cuh -- register-resident FP32 step of the batched service.
//
// One warp owns a work item: a strip of 32 padded columns (28 interior
// columns plus a 2-column halo on each side) of one simulation, over a band
// of H rows.  Lane l holds column i0 + l and marches down the band: each new
// row is loaded once (coalesced), converted to primitives and kept in a
// 4-row register window; x neighbours come from warp shuffles, y neighbours
// from the window.  Every face is solved once (x faces in the lane on their
// right, y faces as the march crosses them), so the step needs no shared
// memory, no barriers and little index arithmetic.  Same physics and update
// order as batch_kernel.cuh (States.h:32-43, RiemannSolvers.h:7-128,
// Update.h:93-174, ThermalConduction.h:36-108, Viscosity.h:27-119), and the
// same per-simulation commit of the step (ComputeDt.h:64, main.cpp:62-83).
#pragma once

#include "batch_common.cuh"
#include "physics.cuh"

namespace fv2d {

namespace bm {

constexpr int STRIP = 28;  // interior columns per warp

__device__ __forceinline__ S4<float> shfl_up4(const S4<float> &q, int d) {
  return S4<float>{__shfl_up_sync(0xffffffffu, q.r, d), __shfl_up_sync(0xffffffffu, q.u, d),
                   __shfl_up_sync(0xffffffffu, q.v, d), __shfl_up_sync(0xffffffffu, q.p, d)};
}
__device__ __forceinline__ S4<float> shfl_down4(const S4<float> &q, int d) {
  return S4<float>{__shfl_down_sync(0xffffffffu, q.r, d), __shfl_down_sync(0xffffffffu, q.u, d),
                   __shfl_down_sync(0xffffffffu, q.v, d), __shfl_down_sync(0xffffffffu, q.p, d)};
}
__device__ __forceinline__ S4<float> add4(const S4<float> &a, const S4<float> &b) {
  return S4<float>{a.r + b.r, a.u + b.u, a.v + b.v, a.p + b.p};
}
__device__ __forceinline__ S4<float> sub4(const S4<float> &a, const S4<float> &b) {
  return S4<float>{a.r - b.r, a.u - b.u, a.v - b.v, a.p - b.p};
}
// half minmod slope of the middle state
__device__ __forceinline__ S4<float> half_slope(const S4<float> &m, const S4<float> &c, const S4<float> &p) {
  return S4<float>{minmod(c.r - m.r, p.r - c.r) * 0.5f, minmod(c.u - m.u, p.u - c.u) * 0.5f,
                   minmod(c.v - m.v, p.v - c.v) * 0.5f, minmod(c.p - m.p, p.p - c.p) * 0.5f};
}

struct SimView {
  const float *src;
  float *dst;
  long long PL;
  int N, P, cur;
  float dt, gamma, gm1, entho, inv_dx, inv_dy, gx, gy, kappa, mu;
  int rs, plm, bcx, bcy, grav, tc, visc, lowmach;
};

// consToPrim with the negative reset (States.h:32-43, SimInfo.h:618-627)
__device__ __forceinline__ S4<float> to_prim(const float u[4], const SimView &S) {
  float r = u[0];
  const float uu = u[1] / r, vv = u[2] / r;
  float p = pressure_of(u[3], r, uu, vv, S.gm1, S.lowmach);
  if (r < 0.f) r = 1e-8f;
  if (p < 0.f) p = 1e-8f;
  return S4<float>{r, uu, vv, p};
}

template <int RS>
__device__ __forceinline__ void solve(const S4<float> &qL, const S4<float> &qR, S4<float> &f, const Gas<float> &gas) {
  float pout;
  if constexpr (RS == RS_HLL)
    riemann_hll(qL, qR, f, pout, gas);
  else
    riemann_hllc(qL, qR, f, pout, gas);
}

// y face between a cell and the one below it (swap_component, States.h:104-110)
template <int RS>
__device__ __forceinline__ S4<float> yflux(const S4<float> &top, const S4<float> &bottom, const Gas<float> &gas) {
  S4<float> f;
  solve<RS>(S4<float>{top.r, top.v, top.u, top.p}, S4<float>{bottom.r, bottom.v, bottom.u, bottom.p}, f, gas);
  return S4<float>{f.r, f.v, f.u, f.p};
}

}  // namespace bm

// One work item (see the header comment), with the Riemann solver and the
// reconstruction fixed at compile time: the kernel dispatches on them once per
// item, so the row loop carries neither branch.
template <int H, int RS, bool PLM>
__device__ __forceinline__ void march_item(const BatchArgs &a, const WorkItem item, const volatile SimDev *G,
                                           const int lane) {
  using namespace bm;
  SimView S;
  S.cur = G->cur;
  S.src = const_cast<const float *>(G->U[S.cur]);
  S.dst = const_cast<float *>(G->U[1 - S.cur]);
  S.PL = G->plane;
  S.N = G->N;
  S.P = G->pitch;
  S.dt = (float)G->dt;
  S.gamma = G->gamma;
  S.gm1 = G->gm1;
  S.entho = G->entho;
  S.inv_dx = G->inv_dx;
  S.inv_dy = G->inv_dy;
  S.gx = G->gx;
  S.gy = G->gy;
  S.kappa = G->kappa;
  S.mu = G->mu;
  S.rs = RS;
  S.plm = PLM;
  S.bcx = G->bcx;
  S.bcy = G->bcy;
  S.grav = G->grav;
  S.tc = G->tc;
  S.visc = G->visc;
  S.lowmach = G->lowmach;
  const Gas<float> gas{S.gamma, S.gm1, S.entho, 1.1f};
  const int N = S.N;
  const int gxl = item.tx * STRIP + lane;           // padded column of this lane
  const bool colok = gxl < N + 4;
  const bool out_lane = lane >= 2 && lane < 30 && gxl - 2 < N;
  const int j0 = item.ty * H, jend = min(j0 + H, N);  // interior rows [j0, jend)
  const float dtdx = S.dt * S.inv_dx, dtdy = S.dt * S.inv_dy;

  auto load = [&](int L, float u[4]) {  // padded row L
    const long long g = (long long)L * S.P + gxl;
    if (colok) {
#pragma unroll
      for (int k = 0; k < 4; ++k) u[k] = __ldg(S.src + k * S.PL + g);
    } else {
      u[0] = 1.f; u[1] = 0.f; u[2] = 0.f; u[3] = 1.f;  // never reaches an output lane
    }
  };
  auto yslope = [&](const S4<float> &m, const S4<float> &c, const S4<float> &p) {
    if constexpr (PLM) return half_slope(m, c, p);
    else return S4<float>{0.f, 0.f, 0.f, 0.f};
  };

  // prologue: rows j0 .. j0+3 (padded) -> window for output row C = j0 + 2
  float ua[4], U0[4], Up[4];
  load(j0, ua);
  const S4<float> qa = to_prim(ua, S);
  load(j0 + 1, ua);
  S4<float> qm = to_prim(ua, S);
  load(j0 + 2, U0);
  S4<float> q0 = to_prim(U0, S);
  load(j0 + 3, Up);
  S4<float> qp = to_prim(Up, S);
  const S4<float> hm = yslope(qa, qm, q0);
  S4<float> h0 = yslope(qm, q0, qp);
  S4<float> Gm = yflux<RS>(add4(qm, hm), sub4(q0, h0), gas);

  float lmax = 0.f;
  unsigned nneg = 0, nnan = 0;
  // rows are loaded one iteration ahead of their use: the loads of row
  // C + 3 are in flight while row C is computed
  float Unext[4];
  load(j0 + 4, Unext);
  for (int C = j0 + 2; C < jend + 2; ++C) {
    float Un[4] = {Unext[0], Unext[1], Unext[2], Unext[3]};
    if (C <= jend) load(C + 3, Unext);
    const S4<float> qn = to_prim(Un, S);
    const S4<float> hp = yslope(q0, qp, qn);
    const S4<float> Gp = yflux<RS>(add4(q0, h0), sub4(qp, hp), gas);

    // x faces of row C: lane l solves face l - 1/2
    const S4<float> qW = shfl_up4(q0, 1), qE = shfl_down4(q0, 1);
    S4<float> hx{0.f, 0.f, 0.f, 0.f};
    if constexpr (PLM) hx = half_slope(qW, q0, qE);
    S4<float> Fw;
    solve<RS>(shfl_up4(add4(q0, hx), 1), sub4(q0, hx), Fw, gas);
    const S4<float> Fe = shfl_down4(Fw, 1);

    // update in the reference's order: x flux, x gravity, y flux, y gravity,
    // conduction, viscosity (Update.h:114-168, 176-191)
    float un[4] = {U0[0], U0[1], U0[2], U0[3]};
    un[0] += (Fw.r - Fe.r) * dtdx;
    un[1] += (Fw.u - Fe.u) * dtdx;
    un[2] += (Fw.v - Fe.v) * dtdx;
    un[3] += (Fw.p - Fe.p) * dtdx;
    if (S.grav) {
      un[2] += S.dt * q0.r * S.gx;
      un[3] += S.dt * 0.5f * (Fw.r + Fe.r) * S.gx;
    }
    un[0] += (Gm.r - Gp.r) * dtdy;
    un[1] += (Gm.u - Gp.u) * dtdy;
    un[2] += (Gm.v - Gp.v) * dtdy;
    un[3] += (Gm.p - Gp.p) * dtdy;
    if (S.grav) {
      un[2] += S.dt * q0.r * S.gy;
      un[3] += S.dt * 0.5f * (Gm.r + Gp.r) * S.gy;
    }
    if (S.tc) {
      const float TC = q0.p / q0.r;
      const float TL = __shfl_up_sync(0xffffffffu, TC, 1), TR = __shfl_down_sync(0xffffffffu, TC, 1);
      const float TU = qm.p / qm.r, TD = qp.p / qp.r;
      const float FL = S.kappa * (TC - TL) * S.inv_dx, FR = S.kappa * (TR - TC) * S.inv_dx;
      const float FU = S.kappa * (TC - TU) * S.inv_dy, FD = S.kappa * (TD - TC) * S.inv_dy;
      un[3] += dtdx * (FR - FL) + dtdy * (FD - FU);
    }
    if (S.visc) {
      // 3x3 stencil of velocities: rows C-1, C, C+1 (qm, q0, qp) x lanes -1, 0, +1
      const float odx = S.inv_dx, ody = S.inv_dy, mu = S.mu;
      float u_[3][3], v_[3][3];
      const S4<float> *rows[3] = {&qm, &q0, &qp};
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        u_[r][1] = rows[r]->u;
        v_[r][1] = rows[r]->v;
        u_[r][0] = __shfl_up_sync(0xffffffffu, u_[r][1], 1);
        v_[r][0] = __shfl_up_sync(0xffffffffu, v_[r][1], 1);
        u_[r][2] = __shfl_down_sync(0xffffffffu, u_[r][1], 1);
        v_[r][2] = __shfl_down_sync(0xffffffffu, v_[r][1], 1);
      }
      auto U_ = [&](int dj, int di) { return u_[dj + 1][di + 1]; };
      auto V_ = [&](int dj, int di) { return v_[dj + 1][di + 1]; };
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
          f1 += sign * mu * txx;
          f2 += sign * mu * txy;
          f3 += sign * mu * (txx * qiu + txy * qiv);
        }
        {
          const float qiu = (U_(s, 0) + U_(sm1, 0)) * 0.5f, qiv = (V_(s, 0) + V_(sm1, 0)) * 0.5f;
          const float dudy = ody * (U_(s, 0) - U_(sm1, 0)), dvdy = ody * (V_(s, 0) - V_(sm1, 0));
          const float dudx = 0.25f * odx * (U_(s, 1) - U_(s, -1) + U_(sm1, 1) - U_(sm1, -1));
          const float dvdx = 0.25f * odx * (V_(s, 1) - V_(s, -1) + V_(sm1, 1) - V_(sm1, -1));
          const float tyy = (4.f / 3.f) * dvdy - (2.f / 3.f) * dudx, txy = dvdx + dudy;
          f1 += sign * mu * txy;
          f2 += sign * mu * tyy;
          f3 += sign * mu * (txy * qiu + tyy * qiv);
        }
      }
      un[1] += f1 * S.dt;
      un[2] += f2 * S.dt;
      un[3] += f3 * S.dt;
    }

    if (out_lane) {
      const int i = gxl - 2, j = C - 2;
      const long long g = (long long)C * S.P + gxl;
#pragma unroll
      for (int k = 0; k < 4; ++k) S.dst[k * S.PL + g] = un[k];
      // primitive state of the new cell for the next dt
      float r = un[0], u = un[1] / r, v = un[2] / r;
      float p = pressure_of(un[3], r, u, v, S.gm1, S.lowmach);
      nnan += is_nan_f(r) | is_nan_f(u) | is_nan_f(v) | is_nan_f(p);
      nneg += (r < 0.f) + (p < 0.f);
      if (r < 0.f) r = 1e-8f;
      if (p < 0.f) p = 1e-8f;
      const float cs = sqrtf(p * S.gamma / r);
      const float ih = (cs + fabsf(u)) * S.inv_dx + (cs + fabsf(v)) * S.inv_dy;
      if (ih > lmax) lmax = ih;  // NaN never enters
      // ghost copies (BoundaryConditions.h:82-147, inverse map)
      const bool ex = (i < 2 || i >= N - 2), ey = (j < 2 || j >= N - 2);
      if (ex || ey) {
        int tx[5], ty[5];
        bool nx[5], ny[5];
        tx[0] = i; nx[0] = false;
        ty[0] = j; ny[0] = false;
        const int cx = 1 + (ex ? ghost_targets(i, N, S.bcx, tx + 1, nx + 1) : 0);
        const int cy = 1 + (ey ? ghost_targets(j, N, S.bcy, ty + 1, ny + 1) : 0);
        for (int b = 0; b < cy; ++b)
          for (int c = 0; c < cx; ++c) {
            if (b == 0 && c == 0) continue;
            const long long gg = (long long)(ty[b] + 2) * S.P + (tx[c] + 2);
            S.dst[gg] = un[0];
            S.dst[S.PL + gg] = nx[c] ? -un[1] : un[1];
            S.dst[2 * S.PL + gg] = ny[b] ? -un[2] : un[2];
            S.dst[3 * S.PL + gg] = un[3];
          }
      }
    }

    // advance the window
    qm = q0;
    q0 = qp;
    qp = qn;
    h0 = hp;
    Gm = Gp;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      U0[k] = Up[k];
      Up[k] = Un[k];
    }
  }

  // item reductions and the per-simulation commit
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) lmax = fmaxf(lmax, __shfl_xor_sync(0xffffffffu, lmax, o));
  const unsigned wn = __reduce_add_sync(0xffffffffu, nneg);
  const unsigned wnan = __reduce_add_sync(0xffffffffu, nnan);
  if (lane == 0) {
    SimDev *Gw = a.sims + item.sim;
    atomicMax(&Gw->acc_bits, __float_as_uint(lmax));
    if (wn) atomicAdd(&Gw->negatives, (unsigned long long)wn);
    if (wnan) atomicAdd(&Gw->nan_cells, wnan);
    __threadfence();
    const unsigned t = atomicAdd(&Gw->ticket, 1u);
    if (t == (unsigned)(G->ntx * G->nty) - 1u) {
      // commit this simulation's step (ComputeDt.h:64, main.cpp:62, 83)
      __threadfence();
      volatile SimDev *V = Gw;
      const double ih = (double)__uint_as_float(atomicAdd(&Gw->acc_bits, 0u));
      double m = ih;
      if (m < V->inv_tc) m = V->inv_tc;
      if (m < V->inv_visc) m = V->inv_visc;
      const double dtn = V->cfl / m;
      const double t_new = V->t + V->dt;
      const int step = V->step + 1;
      V->t = t_new;
      V->step = step;
      V->cur = 1 - S.cur;
      V->dt = dtn;
      V->acc_bits = 0u;
      int status = SIM_ACTIVE;
      if (!(dtn > 0.0) || isinf(dtn) || V->nan_cells)  // the NaN / dt guard fails this request only
        status = SIM_FAILED;
      else if (step >= V->max_steps || !(t_new + V->eps < V->tend))
        status = SIM_DONE;
      V->status = status;
      V->nan_cells = 0u;
      __threadfence();
      V->ticket = 0u;
    }
  }
}

template <int H, int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB) batch_march_kernel(const BatchArgs a) {
  using namespace bm;
  const int lane = threadIdx.x & 31;
  const int nwarps = gridDim.x * (NT / 32);
  const int nw = *a.n_work;
  for (int w = blockIdx.x * (NT / 32) + (threadIdx.x >> 5); w < nw; w += nwarps) {
    const WorkItem item = a.work[w];
    // volatile: the table changes between launches (commits, admissions)
    const volatile SimDev *G = a.sims + item.sim;
    if (G->status != SIM_ACTIVE) continue;
    const bool plm = G->recon == 2;
    if (G->rs == RS_HLL) {
      if (plm)
        march_item<H, RS_HLL, true>(a, item, G, lane);
      else
        march_item<H, RS_HLL, false>(a, item, G, lane);
    } else {
      if (plm)
        march_item<H, RS_HLLC, true>(a, item, G, lane);
      else
        march_item<H, RS_HLLC, false>(a, item, G, lane);
    }
    __syncwarp();
  }
}

}  // namespace fv2d
