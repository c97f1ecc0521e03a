// physics.cuh -- pointwise state math and Riemann solvers of the fv2d hydro
// step, for device code (and host code where marked __host__).
//
// Every expression keeps the operand order of the reference so that, built
// with -fmad=false, binary64 results are bit-identical to it:
//   primToCons / consToPrim / speedOfSound   States.h:19-46
//   hll                                      RiemannSolvers.h:7-51
//   hllc                                     RiemannSolvers.h:53-128
//   fslp                                     RiemannSolvers.h:130-171
//   minmod                                   Update.h:77-85
// Differences from the reference are in control flow only: the Riemann
// solvers evaluate their candidate fluxes without data-dependent branches
// and select at the end (same values, no warp divergence), and constants such
// as 1/(gamma-1) are computed once by the caller with the same operation.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "softfp.cuh"

namespace fv2d {

// Division and square root: binary64 on the device goes through the
// integer-pipe routines (same correctly rounded bits as the hardware
// instructions, off the FP64 pipe); binary32 and host code use the operators.
__host__ __device__ __forceinline__ double fv_div(double a, double b) {
#ifdef __CUDA_ARCH__
  return softfp::div_rn(a, b);
#else
  return a / b;
#endif
}
__host__ __device__ __forceinline__ float fv_div(float a, float b) { return a / b; }
// a1 / b and a2 / b (one reciprocal of b on the device)
__host__ __device__ __forceinline__ void fv_div2(double a1, double a2, double b, double &q1, double &q2) {
#ifdef __CUDA_ARCH__
  const double2 q = softfp::div2_rn(a1, a2, b);
  q1 = q.x;
  q2 = q.y;
#else
  q1 = a1 / b;
  q2 = a2 / b;
#endif
}
__host__ __device__ __forceinline__ void fv_div2(float a1, float a2, float b, float &q1, float &q2) {
  q1 = a1 / b;
  q2 = a2 / b;
}
__host__ __device__ __forceinline__ double fv_sqrt(double x) {
#ifdef __CUDA_ARCH__
  return softfp::sqrt_rn(x);
#else
  return sqrt(x);
#endif
}
__host__ __device__ __forceinline__ float fv_sqrt(float x) { return sqrtf(x); }
// Several quotients by one divisor: r = fv_recip(b) once, fv_div_by(a, b, r)
// per dividend (binary64 on the device: the reciprocal word of b is formed
// once; the quotients are the same correctly rounded values as a / b).
__host__ __device__ __forceinline__ uint64_t fv_recip(double b) {
#ifdef __CUDA_ARCH__
  return softfp::recip_of(b);
#else
  (void)b;
  return 0ull;
#endif
}
__host__ __device__ __forceinline__ double fv_div_by(double a, double b, uint64_t r) {
#ifdef __CUDA_ARCH__
  return softfp::div_by(a, b, r);
#else
  (void)r;
  return a / b;
#endif
}
__host__ __device__ __forceinline__ uint64_t fv_recip(float) { return 0ull; }
__host__ __device__ __forceinline__ float fv_div_by(float a, float b, uint64_t) { return a / b; }

// Comparisons, fmin / fmax and scalings by 1/2: on the device, binary64 goes
// through the bit-pattern forms of softfp.cuh (IEEE results, integer pipe).
#ifdef __CUDA_ARCH__
#define FV2D_D(dev, host) return dev
#else
#define FV2D_D(dev, host) return host
#endif
__host__ __device__ __forceinline__ bool fv_gt0(double x) { FV2D_D(softfp::gt0(x), x > 0.0); }
__host__ __device__ __forceinline__ bool fv_lt0(double x) { FV2D_D(softfp::lt0(x), x < 0.0); }
__host__ __device__ __forceinline__ bool fv_ge0(double x) { FV2D_D(softfp::ge0(x), x >= 0.0); }
__host__ __device__ __forceinline__ bool fv_le0(double x) { FV2D_D(softfp::le0(x), x <= 0.0); }
__host__ __device__ __forceinline__ bool fv_lt(double x, double y) { FV2D_D(softfp::lt(x, y), x < y); }
__host__ __device__ __forceinline__ bool fv_lt_abs(double x, double y) {
  FV2D_D(softfp::lt_abs(x, y), fabs(x) < fabs(y));
}
__host__ __device__ __forceinline__ bool fv_prod_neg(double x, double y) {
  FV2D_D(softfp::prod_neg(x, y), x * y < 0.0);
}
__host__ __device__ __forceinline__ double fv_fmax(double x, double y) { FV2D_D(softfp::fmax_nm(x, y), fmax(x, y)); }
__host__ __device__ __forceinline__ double fv_fmin(double x, double y) { FV2D_D(softfp::fmin_nm(x, y), fmin(x, y)); }
__host__ __device__ __forceinline__ double fv_half(double x) { FV2D_D(softfp::half(x), 0.5 * x); }
__host__ __device__ __forceinline__ double fv_mul(double x, double y) { FV2D_D(softfp::mul_rn(x, y), x * y); }
__host__ __device__ __forceinline__ bool fv_isnan(double x) { FV2D_D(softfp::isnan_b(softfp::bits(x)), isnan(x)); }
#undef FV2D_D
__host__ __device__ __forceinline__ bool fv_gt0(float x) { return x > 0.0f; }
__host__ __device__ __forceinline__ bool fv_lt0(float x) { return x < 0.0f; }
__host__ __device__ __forceinline__ bool fv_ge0(float x) { return x >= 0.0f; }
__host__ __device__ __forceinline__ bool fv_le0(float x) { return x <= 0.0f; }
__host__ __device__ __forceinline__ bool fv_lt(float x, float y) { return x < y; }
__host__ __device__ __forceinline__ bool fv_lt_abs(float x, float y) { return fabsf(x) < fabsf(y); }
__host__ __device__ __forceinline__ bool fv_prod_neg(float x, float y) { return x * y < 0.0f; }
__host__ __device__ __forceinline__ float fv_fmax(float x, float y) { return fmaxf(x, y); }
__host__ __device__ __forceinline__ float fv_fmin(float x, float y) { return fminf(x, y); }
__host__ __device__ __forceinline__ float fv_half(float x) { return 0.5f * x; }
__host__ __device__ __forceinline__ float fv_mul(float x, float y) { return x * y; }
__host__ __device__ __forceinline__ bool fv_isnan(float x) { return isnan(x); }

// Products moved from the binary64 pipe to the integer pipes (softfp::mul_rn),
// by group: the step is bound by the binary64 pipe, and moving every product
// would make the integer pipes the bound instead.  FV2D_SOFT_MUL is a mask
// (bit GROUP - 1 set: that group on the integer pipes); the groups are
//   1  HLLC: energies, p gamma, u* numerator, mass and momentum fluxes
//   2  HLLC: rho/2 (u^2 + v^2)
//   3  the update's dt (F_L - F_R) products
//   4  consToPrim: kinetic energy and (E - Ek)(gamma - 1)
//   5  HLLC: rho (u - S)
//   6  HLLC: p* numerator
//   7  HLLC: star state
//   8  HLLC: energy flux
//   9  HLL: products of each side's state (kinetic energy, fluxes, momenta)
//  10  HLL: the HLL average's products by the wave speeds
//  11  viscous face terms
//  12  conduction fluxes and the conduction / viscosity update products
//  13  MUSCL-Hancock predictor
//  14  FSLP
// The default set measured fastest on the Sedov step.
#ifndef FV2D_SOFT_MUL
#define FV2D_SOFT_MUL 4365
#endif
template <int GROUP, class R>
__host__ __device__ __forceinline__ R mulx(R a, R b) {
  if constexpr ((FV2D_SOFT_MUL >> (GROUP - 1)) & 1) return fv_mul(a, b);
  else return a * b;
}

enum { IR = 0, IU = 1, IV = 2, IP = 3, IE = 3 };

template <class R>
struct S4 {
  R r, u, v, p;  // (rho, u, v, p) or (rho, rho u, rho v, E)
};

// Per-simulation constants used by the pointwise functions.
template <class R>
struct Gas {
  R gamma;   // gamma0
  R gm1;     // gamma0 - 1.0
  R entho;   // 1.0 / (gamma0 - 1.0)               (RiemannSolvers.h:76)
  R fslp_K;  // FSLP K                              (SimInfo.h:399)
  uint64_t rgm1;  // fv_recip(gm1): the divisions by gamma0 - 1 (set by make_gas)
};

template <class R>
__host__ __device__ __forceinline__ Gas<R> make_gas(R gamma, R gm1, R entho, R fslp_K) {
  return Gas<R>{gamma, gm1, entho, fslp_K, fv_recip(gm1)};
}

// States.h:19-30
template <class R>
__host__ __device__ __forceinline__ S4<R> prim_to_cons(const S4<R> &q, const Gas<R> &g) {
  S4<R> s;
  s.r = q.r;
  s.u = q.r * q.u;
  s.v = q.r * q.v;
  R Ek = fv_div(fv_half(s.u * s.u + s.v * s.v), q.r);
  s.p = (Ek + fv_div_by(q.p, g.gm1, g.rgm1));
  return s;
}

// States.h:32-43
template <class R>
__host__ __device__ __forceinline__ S4<R> cons_to_prim(const S4<R> &u, const Gas<R> &g) {
  S4<R> q;
  q.r = u.r;
  fv_div2(u.u, u.v, u.r, q.u, q.v);
  R Ek = mulx<4>(fv_half(q.r), mulx<4>(q.u, q.u) + mulx<4>(q.v, q.v));
  q.p = mulx<4>(u.p - Ek, g.gm1);
  return q;
}

template <class R>
__device__ __forceinline__ R dsqrt(R x) {
  return fv_sqrt(x);
}

// States.h:45-46
template <class R>
__device__ __forceinline__ R sound_speed(const S4<R> &q, const Gas<R> &g) {
  return dsqrt(fv_div(mulx<1>(q.p, g.gamma), q.r));
}
// the same with the reciprocal of q.r already formed (fv_recip)
template <class R>
__device__ __forceinline__ R sound_speed_r(const S4<R> &q, const Gas<R> &g, uint64_t rr) {
  return dsqrt(fv_div_by(mulx<1>(q.p, g.gamma), q.r, rr));
}

// Update.h:77-85
template <class R>
__host__ __device__ __forceinline__ R minmod(R dL, R dR) {
  R m = fv_lt_abs(dL, dR) ? dL : dR;
  return fv_prod_neg(dL, dR) ? R(0) : m;
}

template <class R>
__device__ __forceinline__ R sel(bool c, R a, R b) {
  return c ? a : b;
}

// RiemannSolvers.h:7-51.  All three candidates are evaluated, then selected
// in the reference's branch order (SL >= 0, SR <= 0, else the HLL state).
template <class R>
__device__ __forceinline__ void riemann_hll(const S4<R> &qL, const S4<R> &qR, S4<R> &f, R &pout, const Gas<R> &g) {
  // every quotient by rho_L (rho_R) shares one reciprocal
  const uint64_t rL = fv_recip(qL.r), rR = fv_recip(qR.r);
  const R aL = sound_speed_r(qL, g, rL);
  const R aR = sound_speed_r(qR, g, rR);
  const R sminL = qL.u - aL;
  const R smaxL = qL.u + aL;
  const R sminR = qR.u - aR;
  const R smaxR = qR.u + aR;
  const R SL = fv_fmin(sminL, sminR);
  const R SR = fv_fmax(smaxL, smaxR);
  // computeFlux (RiemannSolvers.h:133-141).  p/(gamma-1) is also the pressure
  // term of primToCons below: the same division, evaluated once.
  const R peL = fv_div_by(qL.p, g.gm1, g.rgm1);
  const R peR = fv_div_by(qR.p, g.gm1, g.rgm1);
  const R EkL = mulx<9>(fv_half(qL.r), mulx<9>(qL.u, qL.u) + mulx<9>(qL.v, qL.v));
  const R EkR = mulx<9>(fv_half(qR.r), mulx<9>(qR.u, qR.u) + mulx<9>(qR.v, qR.v));
  const R EL = (peL + EkL);
  const R ER = (peR + EkR);
  const R ruL = mulx<9>(qL.r, qL.u), ruR = mulx<9>(qR.r, qR.u);
  S4<R> FL{ruL, mulx<9>(ruL, qL.u) + qL.p, mulx<9>(ruL, qL.v), mulx<9>(qL.p + EL, qL.u)};
  S4<R> FR{ruR, mulx<9>(ruR, qR.u) + qR.p, mulx<9>(ruR, qR.v), mulx<9>(qR.p + ER, qR.u)};
  // primToCons (States.h:19-30) of both states
  const R mvL = mulx<9>(qL.r, qL.v), mvR = mulx<9>(qR.r, qR.v);
  const R uEL = (fv_div_by(fv_half(mulx<9>(ruL, ruL) + mulx<9>(mvL, mvL)), qL.r, rL) + peL);
  const R uER = (fv_div_by(fv_half(mulx<9>(ruR, ruR) + mulx<9>(mvR, mvR)), qR.r, rR) + peR);
  const R SLSR = mulx<10>(SL, SR);
  const R den = SR - SL;
  const uint64_t rden = fv_recip(den);
  S4<R> FM;
  FM.r = fv_div_by(mulx<10>(SR, FL.r) - mulx<10>(SL, FR.r) + mulx<10>(SLSR, qR.r - qL.r), den, rden);
  FM.u = fv_div_by(mulx<10>(SR, FL.u) - mulx<10>(SL, FR.u) + mulx<10>(SLSR, ruR - ruL), den, rden);
  FM.v = fv_div_by(mulx<10>(SR, FL.v) - mulx<10>(SL, FR.v) + mulx<10>(SLSR, mvR - mvL), den, rden);
  FM.p = fv_div_by(mulx<10>(SR, FL.p) - mulx<10>(SL, FR.p) + mulx<10>(SLSR, uER - uEL), den, rden);
  const R pM = fv_half(qL.p + qR.p);
  const bool left = fv_ge0(SL);
  const bool right = !left && fv_le0(SR);
  f.r = left ? FL.r : (right ? FR.r : FM.r);
  f.u = left ? FL.u : (right ? FR.u : FM.u);
  f.v = left ? FL.v : (right ? FR.v : FM.v);
  f.p = left ? FL.p : (right ? FR.p : FM.p);
  pout = left ? qL.p : (right ? qR.p : pM);
}

// RiemannSolvers.h:53-128.  The star state is evaluated once, for the side
// the reference would pick if it reaches the star branches (uS > 0 -> left,
// otherwise right), then the final state is chosen in the reference's order.
template <class R>
__device__ __forceinline__ void riemann_hllc(const S4<R> &qL, const S4<R> &qR, S4<R> &f, R &pout, const Gas<R> &g) {
  const R rL = qL.r, uL = qL.u, vL = qL.v, pL = qL.p;
  const R rR = qR.r, uR = qR.u, vR = qR.v, pR = qR.p;
  const R ekL = mulx<2>(fv_half(rL), mulx<1>(uL, uL) + mulx<1>(vL, vL));
  const R EL = ekL + mulx<1>(pL, g.entho);
  const R ekR = mulx<2>(fv_half(rR), mulx<1>(uR, uR) + mulx<1>(vR, vR));
  const R ER = ekR + mulx<1>(pR, g.entho);
  const R cL = sound_speed(qL, g);
  const R cR = sound_speed(qR, g);
  const R cmax = fv_fmax(cL, cR);
  const R SL = fv_fmin(uL, uR) - cmax;
  const R SR = fv_fmax(uL, uR) + cmax;
  const R rcL = mulx<5>(rL, uL - SL);
  const R rcR = mulx<5>(rR, SR - uR);
  R uS, pS;
  fv_div2(mulx<1>(rcR, uR) + mulx<1>(rcL, uL) + (pL - pR),
          mulx<6>(rcR, pL) + mulx<6>(rcL, pR) + mulx<6>(mulx<6>(rcL, rcR), uL - uR), rcR + rcL, uS, pS);
  const bool sideL = fv_gt0(uS);
  const R rK = sideL ? rL : rR;
  const R uK = sideL ? uL : uR;
  const R pK = sideL ? pL : pR;
  const R EK = sideL ? EL : ER;
  const R SK = sideL ? SL : SR;
  R rS, ES;
  fv_div2(mulx<7>(rK, SK - uK), mulx<7>(SK - uK, EK) - mulx<7>(pK, uK) + mulx<7>(pS, uS), SK - uS, rS, ES);
  // branch order of RiemannSolvers.h:89-112
  const bool bL = fv_gt0(SL);
  const bool bStar = !bL && (sideL || fv_gt0(SR));
  R sr, su, sv, sp, E;
  if (bL) {
    sr = rL; su = uL; sv = vL; sp = pL; E = EL;
  } else if (bStar) {
    sr = rS; su = uS; sv = sideL ? vL : vR; sp = pS; E = ES;
  } else {
    sr = rR; su = uR; sv = vR; sp = pR; E = ER;
  }
  pout = sp;
  f.r = mulx<1>(sr, su);
  f.u = mulx<1>(mulx<1>(sr, su), su) + sp;
  f.v = mulx<1>(f.r, sv);
  f.p = mulx<8>(E + sp, su);
}

// RiemannSolvers.h:130-171 (Kokkos::max / min as (a<b)?b:a and (b<a)?b:a).
template <class R>
__device__ __forceinline__ void riemann_fslp(const S4<R> &qL, const S4<R> &qR, S4<R> &f, R &pout, R gdx,
                                             const Gas<R> &g) {
  const R rhoL = qL.r, uL = qL.u, pL = qL.p;
  const R csL = dsqrt(fv_div(mulx<14>(g.gamma, pL), rhoL));
  const R rhoR = qR.r, uR = qR.u, pR = qR.p;
  const R csR = dsqrt(fv_div(mulx<14>(g.gamma, pR), rhoR));
  const R zL = mulx<14>(rhoL, csL), zR = mulx<14>(rhoR, csR);
  const R ai = mulx<14>(g.fslp_K, fv_lt(zL, zR) ? zR : zL);
  const R mL = fv_div(fabs(uL), csL), mR = fv_div(fabs(uR), csR);
  const R mx = fv_lt(mL, mR) ? mR : mL;
  const R theta = fv_lt(mx, R(1)) ? mx : R(1);
  const R ustar = fv_half(uR + uL) - mulx<14>(fv_div(R(0.5), ai), pR - pL - mulx<14>(fv_half(rhoL + rhoR), gdx));
  const R Pi = fv_half(pR + pL) - mulx<14>(mulx<14>(fv_half(theta), ai), uR - uL);
  const bool up = fv_gt0(ustar);
  const R sr = up ? qL.r : qR.r;
  const R su = up ? qL.u : qR.u;
  const R sv = up ? qL.v : qR.v;
  const R sp = up ? qL.p : qR.p;
  const R Ekstar = mulx<14>(fv_half(sr), mulx<14>(su, su) + mulx<14>(sv, sv));
  const R Estar = Ekstar + fv_div_by(sp, g.gm1, g.rgm1);
  const R usr = mulx<14>(ustar, sr);
  f.r = usr;
  f.u = mulx<14>(usr, su) + Pi;
  f.v = mulx<14>(usr, sv);
  f.p = mulx<14>(ustar, Estar + Pi);
  pout = Pi;
}

enum { RS_HLL = 0, RS_HLLC = 1, RS_FSLP = 2 };

template <int RS, class R>
__device__ __forceinline__ void riemann(const S4<R> &qL, const S4<R> &qR, S4<R> &f, R &pout, R gdx, const Gas<R> &g) {
  if constexpr (RS == RS_HLL)
    riemann_hll(qL, qR, f, pout, g);
  else if constexpr (RS == RS_FSLP)
    riemann_fslp(qL, qR, f, pout, gdx, g);
  else
    riemann_hllc(qL, qR, f, pout, g);
}

// Extension (no reference counterpart): primitive-variable MUSCL-Hancock
// half-step qh = q - (dt/2dx) A(q) sx - (dt/2dy) B(q) sy, with ax = 0.5 dt/dx,
// ay = 0.5 dt/dy and sx, sy the full minmod slopes.
template <class R>
__host__ __device__ __forceinline__ S4<R> hancock(const S4<R> &q, const S4<R> &sx, const S4<R> &sy, R ax, R ay,
                                                  R gamma) {
  S4<R> h;
  h.r = q.r - (mulx<13>(ax, mulx<13>(q.u, sx.r) + mulx<13>(q.r, sx.u)) +
               mulx<13>(ay, mulx<13>(q.v, sy.r) + mulx<13>(q.r, sy.v)));
  h.u = q.u - (mulx<13>(ax, mulx<13>(q.u, sx.u) + fv_div(sx.p, q.r)) + mulx<13>(ay, mulx<13>(q.v, sy.u)));
  h.v = q.v - (mulx<13>(ax, mulx<13>(q.u, sx.v)) + mulx<13>(ay, mulx<13>(q.v, sy.v) + fv_div(sy.p, q.r)));
  h.p = q.p - (mulx<13>(ax, mulx<13>(mulx<13>(gamma, q.p), sx.u) + mulx<13>(q.u, sx.p)) +
               mulx<13>(ay, mulx<13>(mulx<13>(gamma, q.p), sy.v) + mulx<13>(q.v, sy.p)));
  return h;
}

// ---------------------------------------------------------------- boundaries
// Source (interior index, 0-based) of ghost `k` along one axis of length N,
// for the boundary fills of BoundaryConditions.h:13-71.  Ghost indices are
// interior-relative: -2, -1 on the low side, N, N+1 on the high side.
// Returns the source index and sets *neg when the normal velocity flips
// (reflecting walls).
__host__ __device__ __forceinline__ int ghost_source(int k, int N, int bc, bool *neg) {
  *neg = false;
  if (k < 0) {
    if (bc == 1) {  // reflecting: 2*ibeg - i - 1
      *neg = true;
      return -k - 1;
    }
    if (bc == 2) return k + N;  // periodic
    return 0;                   // absorbing: copy ibeg
  }
  if (bc == 1) {
    *neg = true;
    return 2 * N - k - 1;
  }
  if (bc == 2) return k - N;
  return N - 1;
}

// Ghost positions (interior-relative) whose source is interior index s;
// returns their count (<= 4) in out[], with the matching negation flags.
__host__ __device__ __forceinline__ int ghost_targets(int s, int N, int bc, int out[4], bool neg[4]) {
  const int ks[4] = {-2, -1, N, N + 1};
  int n = 0;
  for (int t = 0; t < 4; ++t) {
    bool ng;
    if (ghost_source(ks[t], N, bc, &ng) == s) {
      out[n] = ks[t];
      neg[n] = ng;
      ++n;
    }
  }
  return n;
}

}  // namespace fv2d
