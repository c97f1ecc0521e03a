// batch_march2.cuh -- the plain and diffusive families of the served FP32
// step with two columns per lane and packed binary32 arithmetic.
//
// Same work decomposition as batch_march.cuh, but a warp owns a strip of 64
// padded columns (60 interior columns plus the 2-column halo on each side) and
// lane l holds columns 2l and 2l + 1 as the two halves of float2 registers.
// Both columns run the same instructions, so every binary32 add, multiply and
// multiply-add of the step is issued once for the pair (sm_100 packed
// FADD2 / FMUL2 / FFMA2: the one-column body is bound by instruction issue,
// not by the FMA pipe); selects, comparisons, min / max, reciprocals and
// square roots stay per column.  The pair also halves the warp shuffles per
// cell (a column's left or right neighbour is in the same lane half the
// time), the 64-bit loads and stores halve the memory instructions, and the
// halo is 4 of 64 columns instead of 4 of 32.
//
// Physics and update order are those of the one-column kernel (States.h:32-43,
// RiemannSolvers.h:7-128, Update.h:93-174 with constant gravity,
// ThermalConduction.h:36-73 with constant conductivity, Viscosity.h:27-119):
// HLL or HLLC, PCM or PLM.  Each face is solved once; a face that two bands
// share is solved by both, in code whose every operation is an explicitly
// rounded intrinsic or an exact instruction, so both get the same bits and
// the step stays exactly conservative across lanes, strips and bands.
#pragma once

#include "batch_march.cuh"

namespace fv2d {
namespace bm2 {

using bm::SimView;
using bm::WarpSim;

constexpr int STRIP = 60;  // interior columns per warp

typedef float2 f2;
struct b2 {
  bool x, y;
};

__device__ __forceinline__ f2 F2(float a) { return make_float2(a, a); }
__device__ __forceinline__ f2 operator+(f2 a, f2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ f2 operator*(f2 a, f2 b) { return __fmul2_rn(a, b); }
// a - b = b * (-1) + a: one rounding, one packed instruction
__device__ __forceinline__ f2 operator-(f2 a, f2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }
__device__ __forceinline__ f2 fma2(f2 a, f2 b, f2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ f2 rcp2(f2 a) { return make_float2(__fdividef(1.f, a.x), __fdividef(1.f, a.y)); }
__device__ __forceinline__ f2 sqrt2(f2 a) { return make_float2(sqrtf(a.x), sqrtf(a.y)); }
__device__ __forceinline__ f2 min2(f2 a, f2 b) { return make_float2(fminf(a.x, b.x), fminf(a.y, b.y)); }
__device__ __forceinline__ f2 max2(f2 a, f2 b) { return make_float2(fmaxf(a.x, b.x), fmaxf(a.y, b.y)); }
__device__ __forceinline__ f2 sel2(b2 c, f2 a, f2 b) { return make_float2(c.x ? a.x : b.x, c.y ? a.y : b.y); }
__device__ __forceinline__ b2 gt0(f2 a) { return b2{a.x > 0.f, a.y > 0.f}; }
__device__ __forceinline__ b2 ge0(f2 a) { return b2{a.x >= 0.f, a.y >= 0.f}; }
__device__ __forceinline__ b2 le0(f2 a) { return b2{a.x <= 0.f, a.y <= 0.f}; }

typedef S4<f2> Q2;

__device__ __forceinline__ Q2 sub(const Q2 &a, const Q2 &b) { return Q2{a.r - b.r, a.u - b.u, a.v - b.v, a.p - b.p}; }
__device__ __forceinline__ Q2 zero() { return Q2{F2(0.f), F2(0.f), F2(0.f), F2(0.f)}; }
__device__ __forceinline__ Q2 swap_uv(const Q2 &q) { return Q2{q.r, q.v, q.u, q.p}; }

// Neighbours along x of the pair (columns 2l, 2l + 1): the left one is
// (column 2l - 1 from lane l - 1, column 2l), the right one (column 2l + 1,
// column 2l + 2 from lane l + 1).
__device__ __forceinline__ f2 left(f2 a) { return make_float2(__shfl_up_sync(0xffffffffu, a.y, 1), a.x); }
__device__ __forceinline__ f2 right(f2 a) { return make_float2(a.y, __shfl_down_sync(0xffffffffu, a.x, 1)); }
__device__ __forceinline__ Q2 left(const Q2 &q) { return Q2{left(q.r), left(q.u), left(q.v), left(q.p)}; }
__device__ __forceinline__ Q2 right(const Q2 &q) { return Q2{right(q.r), right(q.u), right(q.v), right(q.p)}; }

// minmod (Update.h:77-85) of each column's left and right differences
__device__ __forceinline__ f2 minmod2(f2 dl, f2 dr) {
  const f2 prod = dl * dr;
  const float mx = fabsf(dl.x) < fabsf(dr.x) ? dl.x : dr.x;
  const float my = fabsf(dl.y) < fabsf(dr.y) ? dl.y : dr.y;
  return make_float2(prod.x < 0.f ? 0.f : mx, prod.y < 0.f ? 0.f : my);
}
__device__ __forceinline__ Q2 slope(const Q2 &dl, const Q2 &dr) {
  return Q2{minmod2(dl.r, dr.r), minmod2(dl.u, dr.u), minmod2(dl.v, dr.v), minmod2(dl.p, dr.p)};
}
// q + half * s (Update.h:25)
__device__ __forceinline__ Q2 face(const Q2 &q, const Q2 &s, f2 half) {
  return Q2{fma2(half, s.r, q.r), fma2(half, s.u, q.u), fma2(half, s.v, q.v), fma2(half, s.p, q.p)};
}

struct Gas2 {
  f2 gamma, entho, half;
};

// RiemannSolvers.h:7-51, every candidate evaluated and selected in the
// reference's branch order, per column.
__device__ __forceinline__ void hll(const Q2 &qL, const Q2 &qR, Q2 &f, f2 &pout, const Gas2 &g) {
  const f2 rrL = rcp2(qL.r), rrR = rcp2(qR.r);
  const f2 aL = sqrt2(qL.p * g.gamma * rrL);
  const f2 aR = sqrt2(qR.p * g.gamma * rrR);
  const f2 SL = min2(qL.u - aL, qR.u - aR);
  const f2 SR = max2(qL.u + aL, qR.u + aR);
  const f2 peL = qL.p * g.entho, peR = qR.p * g.entho;
  const f2 EL = peL + (g.half * qL.r) * fma2(qL.u, qL.u, qL.v * qL.v);
  const f2 ER = peR + (g.half * qR.r) * fma2(qR.u, qR.u, qR.v * qR.v);
  const f2 ruL = qL.r * qL.u, ruR = qR.r * qR.u;
  const Q2 FL{ruL, fma2(ruL, qL.u, qL.p), ruL * qL.v, (qL.p + EL) * qL.u};
  const Q2 FR{ruR, fma2(ruR, qR.u, qR.p), ruR * qR.v, (qR.p + ER) * qR.u};
  const f2 mvL = qL.r * qL.v, mvR = qR.r * qR.v;
  const f2 uEL = fma2(g.half * fma2(ruL, ruL, mvL * mvL), rrL, peL);
  const f2 uER = fma2(g.half * fma2(ruR, ruR, mvR * mvR), rrR, peR);
  const f2 SLSR = SL * SR;
  const f2 rden = rcp2(SR - SL);
  Q2 FM;
  FM.r = fma2(SLSR, qR.r - qL.r, SR * FL.r - SL * FR.r) * rden;
  FM.u = fma2(SLSR, ruR - ruL, SR * FL.u - SL * FR.u) * rden;
  FM.v = fma2(SLSR, mvR - mvL, SR * FL.v - SL * FR.v) * rden;
  FM.p = fma2(SLSR, uER - uEL, SR * FL.p - SL * FR.p) * rden;
  const f2 pM = g.half * (qL.p + qR.p);
  const b2 lf = ge0(SL), rt0 = le0(SR);
  const b2 rt{!lf.x && rt0.x, !lf.y && rt0.y};
  f.r = sel2(lf, FL.r, sel2(rt, FR.r, FM.r));
  f.u = sel2(lf, FL.u, sel2(rt, FR.u, FM.u));
  f.v = sel2(lf, FL.v, sel2(rt, FR.v, FM.v));
  f.p = sel2(lf, FL.p, sel2(rt, FR.p, FM.p));
  pout = sel2(lf, qL.p, sel2(rt, qR.p, pM));
}

// RiemannSolvers.h:53-128: the star state of the side the reference would
// reach (u* > 0 -> left), then the final state in its branch order.
__device__ __forceinline__ void hllc(const Q2 &qL, const Q2 &qR, Q2 &f, f2 &pout, const Gas2 &g) {
  const f2 rL = qL.r, uL = qL.u, vL = qL.v, pL = qL.p;
  const f2 rR = qR.r, uR = qR.u, vR = qR.v, pR = qR.p;
  const f2 EL = fma2(g.half * rL, fma2(uL, uL, vL * vL), pL * g.entho);
  const f2 ER = fma2(g.half * rR, fma2(uR, uR, vR * vR), pR * g.entho);
  const f2 cL = sqrt2(pL * g.gamma * rcp2(rL));
  const f2 cR = sqrt2(pR * g.gamma * rcp2(rR));
  const f2 cmax = max2(cL, cR);
  const f2 SL = min2(uL, uR) - cmax;
  const f2 SR = max2(uL, uR) + cmax;
  const f2 rcL = rL * (uL - SL);
  const f2 rcR = rR * (SR - uR);
  const f2 rd = rcp2(rcR + rcL);
  const f2 uS = (fma2(rcR, uR, rcL * uL) + (pL - pR)) * rd;
  const f2 pS = fma2(rcL * rcR, uL - uR, fma2(rcR, pL, rcL * pR)) * rd;
  const b2 sideL = gt0(uS);
  const f2 rK = sel2(sideL, rL, rR);
  const f2 uK = sel2(sideL, uL, uR);
  const f2 pK = sel2(sideL, pL, pR);
  const f2 EK = sel2(sideL, EL, ER);
  const f2 SK = sel2(sideL, SL, SR);
  const f2 rd2 = rcp2(SK - uS);
  const f2 SKu = SK - uK;
  const f2 rS = (rK * SKu) * rd2;
  const f2 ES = fma2(pS, uS, SKu * EK - pK * uK) * rd2;
  const b2 bL = gt0(SL), sR = gt0(SR);
  const b2 bS{!bL.x && (sideL.x || sR.x), !bL.y && (sideL.y || sR.y)};
  const f2 sr = sel2(bL, rL, sel2(bS, rS, rR));
  const f2 su = sel2(bL, uL, sel2(bS, uS, uR));
  const f2 sv = sel2(bL, vL, sel2(bS, sel2(sideL, vL, vR), vR));
  const f2 sp = sel2(bL, pL, sel2(bS, pS, pR));
  const f2 E = sel2(bL, EL, sel2(bS, ES, ER));
  pout = sp;
  f.r = sr * su;
  f.u = fma2(f.r, su, sp);
  f.v = f.r * sv;
  f.p = (E + sp) * su;
}

template <int RS>
__device__ __forceinline__ Q2 solve(const Q2 &qL, const Q2 &qR, const Gas2 &g, f2 &pout) {
  Q2 f;
  if constexpr (RS == RS_HLL)
    hll(qL, qR, f, pout, g);
  else
    hllc(qL, qR, f, pout, g);
  return f;
}

// pressure_of for the pair (batch_common.cuh); the low-Mach recovery per column
__device__ __forceinline__ f2 pressure2(f2 dE, float bg_e, f2 r, f2 u, f2 v, float gm1, int lowmach) {
  if (lowmach)
    return make_float2(pressure_of(dE.x, bg_e, r.x, u.x, v.x, gm1, 1), pressure_of(dE.y, bg_e, r.y, u.y, v.y, gm1, 1));
  const f2 ek = (F2(0.5f) * r) * fma2(u, u, v * v);
  return ((dE - ek) + F2(bg_e)) * F2(gm1);
}

// consToPrim of a stored offset pair (States.h:32-43) with the negative reset
// of checkNegatives (SimInfo.h:618-627) where the reference's Q carries it
__device__ __forceinline__ Q2 to_prim(const f2 u[4], const SimView &S) {
  f2 r = u[0] + F2(S.bg_r);
  const f2 rr = rcp2(r);
  const f2 uu = u[1] * rr, vv = u[2] * rr;
  f2 p = pressure2(u[3], S.bg_e, r, uu, vv, S.gm1, S.lowmach);
  if (!S.avg) {
    if (r.x < 0.f) r.x = 1e-8f;
    if (r.y < 0.f) r.y = 1e-8f;
    if (p.x < 0.f) p.x = 1e-8f;
    if (p.y < 0.f) p.y = 1e-8f;
  }
  return Q2{r, uu, vv, p};
}

}  // namespace bm2

// One work item of the two-column march.  TCV: the diffusive family's body
// (constant conduction and viscosity); the plain body carries neither.
template <int RS, int RECON, bool TCV>
__device__ __forceinline__ void march2_item(const BatchArgs &a, const WorkItem item, const bm::WarpSim &W,
                                            const int lane) {
  using namespace bm2;
  constexpr bool SLOPES = RECON != BR_PCM;
  SimView S;
  {
    float *U[2] = {bm::sim_get<float *, offsetof(SimDev, U)>(W), bm::sim_get<float *, offsetof(SimDev, U) + 8>(W)};
    const StageBuffers B = stage_buffers(U, FV2D_SIM(W, cur), FV2D_SIM(W, ts), FV2D_SIM(W, stage));
    S.src = B.src;
    S.dst = B.dst;
    S.avg = B.avg;
    S.last = B.last;
  }
  S.PL = FV2D_SIM(W, plane);
  S.Nx = FV2D_SIM(W, Nx);
  S.Ny = FV2D_SIM(W, Ny);
  S.P = FV2D_SIM(W, pitch);
  S.dt = (float)FV2D_SIM(W, dt);
  S.gamma = FV2D_SIM(W, gamma);
  S.gm1 = FV2D_SIM(W, gm1);
  S.inv_dx = FV2D_SIM(W, inv_dx);
  S.inv_dy = FV2D_SIM(W, inv_dy);
  S.gx = FV2D_SIM(W, gx);
  S.gy = FV2D_SIM(W, gy);
  S.kappa = FV2D_SIM(W, kappa);
  S.mu = FV2D_SIM(W, mu);
  S.bg_r = FV2D_SIM(W, bg_r);
  S.bg_e = FV2D_SIM(W, bg_e);
  S.bcx = FV2D_SIM(W, bcx);
  S.bcy = FV2D_SIM(W, bcy);
  S.grav = FV2D_SIM(W, grav);
  S.tc = FV2D_SIM(W, tc);
  S.visc = FV2D_SIM(W, visc);
  S.lowmach = FV2D_SIM(W, lowmach);
  const Gas2 gas{F2(S.gamma), F2(FV2D_SIM(W, entho)), F2(0.5f)};
  const int ntiles = FV2D_SIM(W, ntx) * FV2D_SIM(W, nty);
  const int Nx = S.Nx, Ny = S.Ny;
  const int gxl = item.tx * STRIP + 2 * lane;  // padded column of the pair's first half (even)
  const bool colok = gxl < Nx + 4;             // then gxl + 1 < pitch: the pair lies in the row
  const bool out0 = lane >= 1 && lane < 31 && gxl - 2 < Nx;  // columns 2..61 of the strip are interior
  const bool out1 = out0 && gxl - 1 < Nx;
  const int band = FV2D_SIM(W, band);
  const int j0 = item.ty * band, jend = min(j0 + band, Ny);
  const f2 dtdx = F2(S.dt * S.inv_dx), dtdy = F2(S.dt * S.inv_dy);

  auto load = [&](int L, f2 u[4]) {  // padded row L, columns gxl and gxl + 1
    const long long g = (long long)L * S.P + gxl;
    if (colok) {
#pragma unroll
      for (int k = 0; k < 4; ++k) u[k] = __ldg(reinterpret_cast<const float2 *>(S.src + k * S.PL + g));
    } else {
      u[0] = F2(1.f); u[1] = F2(0.f); u[2] = F2(0.f); u[3] = F2(1.f);  // never reaches an output column
    }
  };
  const Q2 z = zero();
  auto yslope = [&](const Q2 &dl, const Q2 &dr) {
    if constexpr (SLOPES) return slope(dl, dr);
    else return z;
  };
  auto ydiff = [&](const Q2 &lo, const Q2 &hi) {
    if constexpr (SLOPES) return sub(hi, lo);
    else return z;
  };
  // x slope of a row: each column's left difference, the right one from the
  // next column
  auto xslope = [&](const Q2 &c) {
    if constexpr (SLOPES) {
      const Q2 dl = sub(c, left(c));
      return slope(dl, right(dl));
    } else {
      return z;
    }
  };
  const f2 hp5 = F2(0.5f), hm5 = F2(-0.5f);

  // The row loop of batch_march.cuh, with its four window-fill iterations
  // peeled into a prologue so that the main loop's y-face and x-face solves,
  // which are independent, share one block the compiler can interleave.
  // Iteration L loads padded row L and (from L = j0 + 4 on) updates row
  // C = L - 2.  Both copies of the row entry and of the y face are the same
  // functions of the same operands, and every operation in them is an explicit
  // packed intrinsic or an exact instruction (nothing is left for the compiler
  // to contract), so a face that two bands share gets bit-identical fluxes from
  // the prologue of one and the main loop of the other: the step stays exactly
  // conservative.
  // The window carries the primitives of rows L - 2 and L - 1 (q0, qp), the
  // y slope of row L - 2, the y flux of face C - 1/2 and the prefetched next
  // row; the conservative row C is read again at its update (an L1 hit: it
  // was loaded two iterations earlier) and the primitives of row C - 1 are
  // rebuilt from memory only when conduction or viscosity need them.
  Q2 q0 = z, qp = z, h0 = z, Gm = z;
  f2 Unext[4];
  float lmax = 0.f;
  unsigned nneg = 0, nnan = 0;
  // primitives of the new row L and the y slope of row L - 1
  auto enter = [&](const f2 Un[4], Q2 &qn, Q2 &hp) {
    qn = to_prim(Un, S);
    hp = yslope(ydiff(q0, qp), ydiff(qp, qn));
  };
  // y face between rows L - 2 and L - 1
  auto yface = [&](const Q2 &hp) {
    f2 pout;
    return swap_uv(solve<RS>(swap_uv(face(q0, h0, hp5)), swap_uv(face(qp, hp, hm5)), gas, pout));
  };
  load(j0, Unext);
  for (int L = j0; L < j0 + 4; ++L) {  // jend >= j0 + 1: row L + 1 is in the band's window
    const f2 Un[4] = {Unext[0], Unext[1], Unext[2], Unext[3]};
    load(L + 1, Unext);
    Q2 qn, hp;
    enter(Un, qn, hp);
    if (L == j0 + 3) Gm = yface(hp);
    q0 = qp;
    qp = qn;
    h0 = hp;
  }
  for (int L = j0 + 4; L < jend + 4; ++L) {
    const int C = L - 2;
    const int j = C - 2;
    const f2 Un[4] = {Unext[0], Unext[1], Unext[2], Unext[3]};
    if (L + 1 < jend + 4) load(L + 1, Unext);
    Q2 qn, hp;
    enter(Un, qn, hp);
    const Q2 Gp = yface(hp);  // face between rows C and C + 1
    {
      // x faces of row C: the pair solves faces 2l - 1/2 and 2l + 1/2
      const Q2 hx = xslope(q0);
      f2 poutX;
      const Q2 Fw = solve<RS>(left(face(q0, hx, hp5)), face(q0, hx, hm5), gas, poutX);
      const Q2 Fe = right(Fw);

      // update in the reference's order: x flux, x gravity, y flux, y
      // gravity, conduction, viscosity (Update.h:114-168, 176-191)
      f2 un[4], U0[4];
      load(C, U0);
      un[0] = fma2(Fw.r - Fe.r, dtdx, U0[0]);
      un[1] = fma2(Fw.u - Fe.u, dtdx, U0[1]);
      un[2] = fma2(Fw.v - Fe.v, dtdx, U0[2]);
      un[3] = fma2(Fw.p - Fe.p, dtdx, U0[3]);
      const f2 dt2 = F2(S.dt);
      if (S.grav) {
        un[2] = fma2(dt2 * q0.r, F2(S.gx), un[2]);
        un[3] = fma2(dt2 * (hp5 * (Fw.r + Fe.r)), F2(S.gx), un[3]);
      }
      un[0] = fma2(Gm.r - Gp.r, dtdy, un[0]);
      un[1] = fma2(Gm.u - Gp.u, dtdy, un[1]);
      un[2] = fma2(Gm.v - Gp.v, dtdy, un[2]);
      un[3] = fma2(Gm.p - Gp.p, dtdy, un[3]);
      if (S.grav) {
        un[2] = fma2(dt2 * q0.r, F2(S.gy), un[2]);
        un[3] = fma2(dt2 * (hp5 * (Gm.r + Gp.r)), F2(S.gy), un[3]);
      }
      Q2 qm = z;  // primitives of row C - 1
      if (TCV && (S.tc || S.visc)) {
        f2 Um[4];
        load(C - 1, Um);
        qm = to_prim(Um, S);
      }
      if (TCV && S.tc) {  // constant conductivity (ThermalConduction.h:36-73)
        const f2 TC = q0.p * rcp2(q0.r);
        const f2 TL = left(TC), TR = right(TC);
        const f2 TU = qm.p * rcp2(qm.r), TD = qp.p * rcp2(qp.r);
        const f2 kx = F2(S.kappa * S.inv_dx), ky = F2(S.kappa * S.inv_dy);
        const f2 FL = kx * (TC - TL), FR = kx * (TR - TC);
        const f2 FU = ky * (TC - TU), FD = ky * (TD - TC);
        un[3] = un[3] + fma2(dtdx, FR - FL, dtdy * (FD - FU));
      }
      if (TCV && S.visc) {
        // 3x3 stencil of velocities: rows C-1, C, C+1 (qm, q0, qp) x columns -1, 0, +1
        const f2 odx = F2(S.inv_dx), ody = F2(S.inv_dy);
        f2 u_[3][3], v_[3][3];
        const Q2 *rws[3] = {&qm, &q0, &qp};
#pragma unroll
        for (int r = 0; r < 3; ++r) {
          u_[r][1] = rws[r]->u;
          v_[r][1] = rws[r]->v;
          u_[r][0] = left(u_[r][1]);
          v_[r][0] = left(v_[r][1]);
          u_[r][2] = right(u_[r][1]);
          v_[r][2] = right(v_[r][1]);
        }
        auto U_ = [&](int dj, int di) { return u_[dj + 1][di + 1]; };
        auto V_ = [&](int dj, int di) { return v_[dj + 1][di + 1]; };
        const f2 c43 = F2(4.f / 3.f), c23 = F2(2.f / 3.f), q25 = F2(0.25f);
        f2 f1 = F2(0.f), f2_ = F2(0.f), f3 = F2(0.f);
#pragma unroll
        for (int side = 1; side < 3; ++side) {
          const f2 smu = F2(side == 1 ? -S.mu : S.mu);
          const int s = side - 1, sm1 = side - 2;
          {
            const f2 qiu = (U_(0, s) + U_(0, sm1)) * hp5, qiv = (V_(0, s) + V_(0, sm1)) * hp5;
            const f2 dudx = odx * (U_(0, s) - U_(0, sm1)), dvdx = odx * (V_(0, s) - V_(0, sm1));
            const f2 dudy = (q25 * ody) * ((U_(1, s) - U_(-1, s)) + (U_(1, sm1) - U_(-1, sm1)));
            const f2 dvdy = (q25 * ody) * ((V_(1, s) - V_(-1, s)) + (V_(1, sm1) - V_(-1, sm1)));
            const f2 txx = c43 * dudx - c23 * dvdy, txy = dvdx + dudy;
            f1 = fma2(smu, txx, f1);
            f2_ = fma2(smu, txy, f2_);
            f3 = fma2(smu, fma2(txx, qiu, txy * qiv), f3);
          }
          {
            const f2 qiu = (U_(s, 0) + U_(sm1, 0)) * hp5, qiv = (V_(s, 0) + V_(sm1, 0)) * hp5;
            const f2 dudy = ody * (U_(s, 0) - U_(sm1, 0)), dvdy = ody * (V_(s, 0) - V_(sm1, 0));
            const f2 dudx = (q25 * odx) * ((U_(s, 1) - U_(s, -1)) + (U_(sm1, 1) - U_(sm1, -1)));
            const f2 dvdx = (q25 * odx) * ((V_(s, 1) - V_(s, -1)) + (V_(sm1, 1) - V_(sm1, -1)));
            const f2 tyy = c43 * dvdy - c23 * dudx, txy = dvdx + dudy;
            f1 = fma2(smu, txy, f1);
            f2_ = fma2(smu, tyy, f2_);
            f3 = fma2(smu, fma2(txy, qiu, tyy * qiv), f3);
          }
        }
        un[1] = fma2(f1, dt2, un[1]);
        un[2] = fma2(f2_, dt2, un[2]);
        un[3] = fma2(f3, dt2, un[3]);
      }

      if (out0) {
        const long long g = (long long)C * S.P + gxl;
        if (S.avg) {  // SSP-RK2: 0.5 (U^n + U**) (Update.h:214-220), offsets alike
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            const float *d = S.dst + k * S.PL + g;
            const f2 o = out1 ? *reinterpret_cast<const float2 *>(d) : make_float2(d[0], 0.f);
            un[k] = hp5 * (o + un[k]);
          }
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          float *d = S.dst + k * S.PL + g;
          if (out1)
            *reinterpret_cast<float2 *>(d) = un[k];
          else
            d[0] = un[k].x;
        }
        if (S.last) {
          // primitive state of the new cells for the next dt, negative guard
          f2 r = un[0] + F2(S.bg_r);
          const f2 rr = rcp2(r);
          const f2 u = un[1] * rr, v = un[2] * rr;
          f2 p = pressure2(un[3], S.bg_e, r, u, v, S.gm1, S.lowmach);
          const float rx[2] = {r.x, r.y}, ux[2] = {u.x, u.y}, vx[2] = {v.x, v.y}, px[2] = {p.x, p.y};
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            if (h == 1 && !out1) break;
            float rh = rx[h], ph = px[h];
            nnan += is_nan_f(rh) | is_nan_f(ux[h]) | is_nan_f(vx[h]) | is_nan_f(ph);
            nneg += (rh < 0.f) + (ph < 0.f);
            if (rh < 0.f) rh = 1e-8f;
            if (ph < 0.f) ph = 1e-8f;
            const float cs = sqrtf(ph * S.gamma * __fdividef(1.f, rh));
            const float ih = (cs + fabsf(ux[h])) * S.inv_dx + (cs + fabsf(vx[h])) * S.inv_dy;
            if (ih > lmax) lmax = ih;  // NaN never enters
          }
        } else {
          nnan += is_nan_f(un[0].x) | is_nan_f(un[1].x) | is_nan_f(un[2].x) | is_nan_f(un[3].x);
          if (out1) nnan += is_nan_f(un[0].y) | is_nan_f(un[1].y) | is_nan_f(un[2].y) | is_nan_f(un[3].y);
        }
        // ghost copies (BoundaryConditions.h:82-147, inverse map), per column
        const int i0 = gxl - 2;
        const bool ey = (j < 2 || j >= Ny - 2);
        const bool ex = (i0 < 2 || i0 + 1 >= Nx - 2);
        if (ex || ey) {
          const float ur[2] = {un[0].x, un[0].y}, uu[2] = {un[1].x, un[1].y}, uv[2] = {un[2].x, un[2].y},
                      ue[2] = {un[3].x, un[3].y};
          for (int h = 0; h < 2; ++h) {
            if (h == 1 && !out1) break;
            const int i = i0 + h;
            const bool exh = (i < 2 || i >= Nx - 2);
            if (!exh && !ey) continue;
            int tx[5], ty[5];
            bool nx[5], ny[5];
            tx[0] = i; nx[0] = false;
            ty[0] = j; ny[0] = false;
            const int cx = 1 + (exh ? ghost_targets(i, Nx, S.bcx, tx + 1, nx + 1) : 0);
            const int cy = 1 + (ey ? ghost_targets(j, Ny, S.bcy, ty + 1, ny + 1) : 0);
            for (int b = 0; b < cy; ++b)
              for (int c = 0; c < cx; ++c) {
                if (b == 0 && c == 0) continue;
                const long long gg = (long long)(ty[b] + 2) * S.P + (tx[c] + 2);
                S.dst[gg] = ur[h];
                S.dst[S.PL + gg] = nx[c] ? -uu[h] : uu[h];
                S.dst[2 * S.PL + gg] = ny[b] ? -uv[h] : uv[h];
                S.dst[3 * S.PL + gg] = ue[h];
              }
          }
        }
      }
    }

    // advance the window
    q0 = qp;
    qp = qn;
    h0 = hp;
    Gm = Gp;
  }

  // item reductions and the per-simulation commit
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) lmax = fmaxf(lmax, __shfl_xor_sync(0xffffffffu, lmax, o));
  const unsigned wn = __reduce_add_sync(0xffffffffu, nneg);
  const unsigned wnan = __reduce_add_sync(0xffffffffu, nnan);
  if (lane == 0) {
    SimDev *Gw = a.sims + item.sim;
    if (S.last) atomicMax(&Gw->acc_bits, __float_as_uint(lmax));
    if (wn) atomicAdd(&Gw->negatives, (unsigned long long)wn);
    if (wnan) atomicAdd(&Gw->nan_cells, wnan);
    __threadfence();
    const unsigned t = atomicAdd(&Gw->ticket, 1u);
    if (t == (unsigned)ntiles - 1u) commit_stage(Gw);
  }
}

// The plain (TCV false) or diffusive (TCV true) family with two columns per
// lane: HLL / HLLC x PCM / PLM.  A request of the other family never enters
// (the service keeps the families in separate lanes); if one did, it would
// fail rather than run without its conduction and viscosity.
template <int NT, int MINB, bool TCV>
__global__ void __launch_bounds__(NT, MINB) batch_march2_kernel(const BatchArgs a) {
  const int lane = threadIdx.x & 31;
  const int nwarps = gridDim.x * (NT / 32);
  const int nw = *a.n_work;
  for (int w = blockIdx.x * (NT / 32) + (threadIdx.x >> 5); w < nw; w += nwarps) {
    const WorkItem item = a.work[w];
    const bm::WarpSim W = bm::load_sim(a.sims + item.sim, lane);
    if (FV2D_SIM(W, status) != SIM_ACTIVE) continue;
    if (!TCV && (FV2D_SIM(W, tc) || FV2D_SIM(W, visc))) {
      if (lane == 0) {  // fail the request through its commit, like a wait that gave up
        SimDev *Gw = a.sims + item.sim;
        atomicOr(&Gw->dev_err, (unsigned)BATCH_ERR_FAMILY);
        __threadfence();
        const unsigned t = atomicAdd(&Gw->ticket, 1u);
        if (t == (unsigned)(FV2D_SIM(W, ntx) * FV2D_SIM(W, nty)) - 1u) commit_stage(Gw);
      }
      __syncwarp();
      continue;
    }
    const bool plm = FV2D_SIM(W, recon) == BR_PLM;
    if (FV2D_SIM(W, rs) == RS_HLL) {
      if (plm)
        march2_item<RS_HLL, BR_PLM, TCV>(a, item, W, lane);
      else
        march2_item<RS_HLL, BR_PCM, TCV>(a, item, W, lane);
    } else {
      if (plm)
        march2_item<RS_HLLC, BR_PLM, TCV>(a, item, W, lane);
      else
        march2_item<RS_HLLC, BR_PCM, TCV>(a, item, W, lane);
    }
    __syncwarp();
  }
}

}  // namespace fv2d
