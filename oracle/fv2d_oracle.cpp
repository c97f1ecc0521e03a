// fv2d_oracle.cpp -- TEST INFRASTRUCTURE (the oracle), not part of the product.
//
// CPU FP64 restatement of mdelorme/fv2d's explicit hydro step.  Each
// function names the reference lines it restates.  The pass structure and the
// order of every floating-point operation follow the reference; the build
// uses -ffp-contract=off so that no multiply-add is fused.
//
// Storage mirrors the reference's Array(Nty, Ntx, 4) in row-major order
// (Kokkos LayoutRight on host back-ends): element (j, i, v) at
// ((j * Ntx) + i) * 4 + v, ghosts included.
#include "fv2d_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <new>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

using real_t = double;
struct State {
  real_t v[4];
  real_t &operator[](int k) { return v[k]; }
  const real_t &operator[](int k) const { return v[k]; }
};
enum { IR = 0, IU = 1, IV = 2, IP = 3, IE = 3 };
enum Dir { IX = 0, IY = 1 };

// State arithmetic of States.h:48-101 (component-wise, same operand order).
inline State operator+(const State &a, const State &b) {
  State r;
  for (int k = 0; k < 4; ++k) r[k] = a[k] + b[k];
  return r;
}
inline State operator-(const State &a, const State &b) {
  State r;
  for (int k = 0; k < 4; ++k) r[k] = a[k] - b[k];
  return r;
}
inline State operator*(const State &a, real_t q) {
  State r;
  for (int k = 0; k < 4; ++k) r[k] = a[k] * q;
  return r;
}
inline State operator*(real_t q, const State &a) { return a * q; }
inline State operator/(const State &a, real_t q) {
  State r;
  for (int k = 0; k < 4; ++k) r[k] = a[k] / q;
  return r;
}
inline State &operator+=(State &a, const State &b) {
  for (int k = 0; k < 4; ++k) a[k] += b[k];
  return a;
}

// States.h:103-110
inline State swap_component(const State &q, Dir d) {
  if (d == IX) return q;
  return State{{q[IR], q[IV], q[IU], q[IP]}};
}

struct Grid {
  int Nx, Ny, Ng, Ntx, Nty, ibeg, iend, jbeg, jend;
  real_t xmin, xmax, ymin, ymax, dx, dy;
};

int g_threads = 0;

}  // namespace

struct fv2d_oracle {
  fv2d_params p;
  Grid g;
  std::vector<real_t> Q, U, slopesX, slopesY, U0, Ustar;
  uint64_t counters[3] = {0, 0, 0};

  size_t at(int j, int i, int v) const { return ((size_t)j * g.Ntx + i) * 4 + v; }
  State get(const std::vector<real_t> &a, int i, int j) const {  // States.h:6-10
    size_t b = at(j, i, 0);
    return State{{a[b], a[b + 1], a[b + 2], a[b + 3]}};
  }
  void set(std::vector<real_t> &a, int i, int j, const State &s) const {  // States.h:12-17
    size_t b = at(j, i, 0);
    for (int k = 0; k < 4; ++k) a[b + k] = s[k];
  }
};

namespace {

// ---------------------------------------------------------------- States.h
// States.h:19-30
State primToCons(const State &q, const fv2d_params &p) {
  State res;
  res[IR] = q[IR];
  res[IU] = q[IR] * q[IU];
  res[IV] = q[IR] * q[IV];
  real_t Ek = 0.5 * (res[IU] * res[IU] + res[IV] * res[IV]) / q[IR];
  res[IE] = (Ek + q[IP] / (p.gamma0 - 1.0));
  return res;
}

// States.h:32-43
State consToPrim(const State &u, const fv2d_params &p) {
  State res;
  res[IR] = u[IR];
  res[IU] = u[IU] / u[IR];
  res[IV] = u[IV] / u[IR];
  real_t Ek = 0.5 * res[IR] * (res[IU] * res[IU] + res[IV] * res[IV]);
  res[IP] = (u[IE] - Ek) * (p.gamma0 - 1.0);
  return res;
}

// States.h:45-46
real_t speedOfSound(const State &q, const fv2d_params &p) { return std::sqrt(q[IP] * p.gamma0 / q[IR]); }

// SimInfo.h:494-499
inline real_t posX(const Grid &g, int i) { return g.xmin + (i - g.ibeg + 0.5) * g.dx; }
inline real_t posY(const Grid &g, int j) { return g.ymin + (j - g.jbeg + 0.5) * g.dy; }

// ---------------------------------------------------------------- Gravity.h
// Gravity.h:15-28 (the value is narrowed to float on return)
float analyticalGravity(const Grid &g, const fv2d_params &p, int /*i*/, int j) {
  real_t y = posY(g, j);
  real_t gv = p.hot_bubble_g0 * std::sin(y * M_PI * 2.0 / p.ymax);
  return (float)gv;
}
// Gravity.h:30-57
float getGravity(const Grid &g, const fv2d_params &p, int i, int j, Dir d) {
  real_t gv;
  switch (p.gravity_mode) {
    case FV2D_GRAV_CONSTANT: gv = (d == IX ? p.gx : p.gy); break;
    case FV2D_GRAV_ANALYTICAL: gv = analyticalGravity(g, p, i, j); break;
    default: gv = 0.0; break;
  }
  return (float)gv;
}

// ---------------------------------------------------------------- RiemannSolvers.h
// RiemannSolvers.h:7-51
void hll(const State &qL, const State &qR, State &flux, real_t &pout, const fv2d_params &p) {
  const real_t aL = speedOfSound(qL, p);
  const real_t aR = speedOfSound(qR, p);
  const real_t sminL = qL[IU] - aL;
  const real_t smaxL = qL[IU] + aL;
  const real_t sminR = qR[IU] - aR;
  const real_t smaxR = qR[IU] + aR;
  const real_t SL = std::fmin(sminL, sminR);
  const real_t SR = std::fmax(smaxL, smaxR);
  auto computeFlux = [&](const State &q) {
    const real_t Ek = 0.5 * q[IR] * (q[IU] * q[IU] + q[IV] * q[IV]);
    const real_t E = (q[IP] / (p.gamma0 - 1.0) + Ek);
    return State{{q[IR] * q[IU], q[IR] * q[IU] * q[IU] + q[IP], q[IR] * q[IU] * q[IV], (q[IP] + E) * q[IU]}};
  };
  State FL = computeFlux(qL);
  State FR = computeFlux(qR);
  if (SL >= 0.0) {
    flux = FL;
    pout = qL[IP];
  } else if (SR <= 0.0) {
    flux = FR;
    pout = qR[IP];
  } else {
    State uL = primToCons(qL, p);
    State uR = primToCons(qR, p);
    pout = 0.5 * (qL[IP] + qR[IP]);
    flux = (SR * FL - SL * FR + SL * SR * (uR - uL)) / (SR - SL);
  }
}

// RiemannSolvers.h:53-128
void hllc(const State &qL, const State &qR, State &flux, real_t &pout, const fv2d_params &p) {
  const real_t rL = qL[IR], uL = qL[IU], vL = qL[IV], pL = qL[IP];
  const real_t rR = qR[IR], uR = qR[IU], vR = qR[IV], pR = qR[IP];
  const real_t entho = 1.0 / (p.gamma0 - 1.0);
  const real_t ekL = 0.5 * rL * (uL * uL + vL * vL);
  const real_t EL = ekL + pL * entho;
  const real_t ekR = 0.5 * rR * (uR * uR + vR * vR);
  const real_t ER = ekR + pR * entho;
  const real_t cfastL = speedOfSound(qL, p);
  const real_t cfastR = speedOfSound(qR, p);
  const real_t SL = std::fmin(uL, uR) - std::fmax(cfastL, cfastR);
  const real_t SR = std::fmax(uL, uR) + std::fmax(cfastL, cfastR);
  const real_t rcL = rL * (uL - SL);
  const real_t rcR = rR * (SR - uR);
  const real_t uS = (rcR * uR + rcL * uL + (pL - pR)) / (rcR + rcL);
  const real_t pS = (rcR * pL + rcL * pR + rcL * rcR * (uL - uR)) / (rcR + rcL);
  const real_t rSL = rL * (SL - uL) / (SL - uS);
  const real_t ESL = ((SL - uL) * EL - pL * uL + pS * uS) / (SL - uS);
  const real_t rSR = rR * (SR - uR) / (SR - uS);
  const real_t ESR = ((SR - uR) * ER - pR * uR + pS * uS) / (SR - uS);
  State st;
  real_t E;
  if (SL > 0.0) {
    st = qL;
    E = EL;
    pout = pL;
  } else if (uS > 0.0) {
    st = State{{rSL, uS, qL[IV], pS}};
    E = ESL;
    pout = pS;
  } else if (SR > 0.0) {
    st = State{{rSR, uS, qR[IV], pS}};
    E = ESR;
    pout = pS;
  } else {
    st = qR;
    E = ER;
    pout = pR;
  }
  flux[IR] = st[IR] * st[IU];
  flux[IU] = st[IR] * st[IU] * st[IU] + st[IP];
  flux[IV] = flux[IR] * st[IV];
  flux[IE] = (E + st[IP]) * st[IU];
}

// RiemannSolvers.h:130-171 (Kokkos::max/min/abs restated as ternaries)
inline real_t kmax(real_t a, real_t b) { return (a < b) ? b : a; }
inline real_t kmin(real_t a, real_t b) { return (b < a) ? b : a; }
void fslp(const State &qL, const State &qR, State &flux, real_t &pout, real_t gdx, const fv2d_params &p) {
  const real_t rhoL = qL[IR], uL = qL[IU], pL = qL[IP];
  const real_t csL = std::sqrt(p.gamma0 * pL / rhoL);
  const real_t rhoR = qR[IR], uR = qR[IU], pR = qR[IP];
  const real_t csR = std::sqrt(p.gamma0 * pR / rhoR);
  const real_t ai = p.fslp_K * kmax(rhoL * csL, rhoR * csR);
  const real_t theta = kmin(1.0, kmax(std::fabs(uL) / csL, std::fabs(uR) / csR));
  const real_t ustar = 0.5 * (uR + uL) - 0.5 / ai * (pR - pL - 0.5 * (rhoL + rhoR) * gdx);
  const real_t Pi = 0.5 * (pR + pL) - theta * 0.5 * ai * (uR - uL);
  const State &qs = (ustar > 0 ? qL : qR);
  const real_t Ekstar = 0.5 * qs[IR] * (qs[IU] * qs[IU] + qs[IV] * qs[IV]);
  const real_t Estar = Ekstar + qs[IP] / (p.gamma0 - 1.0);
  flux[IR] = ustar * qs[IR];
  flux[IU] = ustar * qs[IR] * qs[IU] + Pi;
  flux[IV] = ustar * qs[IR] * qs[IV];
  flux[IE] = ustar * (Estar + Pi);
  pout = Pi;
}

// ---------------------------------------------------------------- ThermalConduction.h / Viscosity.h
// ThermalConduction.h:8-26.  The reference also calls this with real
// coordinates converted to int (ThermalConduction.h:50-53); callers pass the
// converted values.
real_t computeKappa(const Grid &g, const fv2d_params &p, int /*i*/, int j) {
  if (p.thermal_conductivity_mode == FV2D_TCM_B02) {
    const real_t y = posY(g, j);
    const real_t tr = (std::tanh((y - p.b02_ymid) / p.b02_thickness) + 1.0) * 0.5;
    return p.kappa * (p.b02_kappa1 * (1.0 - tr) + p.b02_kappa2 * tr);
  }
  return p.kappa;
}
// Viscosity.h:8-17
real_t computeMu(const fv2d_params &p) { return p.mu; }

// ---------------------------------------------------------------- extension: MUSCL-Hancock predictor
// Not in the reference.  Primitive-variable half-step
//   qh = q - (dt/2dx) A(q) dqx - (dt/2dy) B(q) dqy
// with the Euler primitive Jacobians; the GPU kernels use the identical
// operation order.
State hancock(const State &q, const State &sx, const State &sy, real_t ax, real_t ay, real_t gamma0) {
  const real_t r = q[IR], u = q[IU], v = q[IV], pr = q[IP];
  State h;
  h[IR] = r - (ax * (u * sx[IR] + r * sx[IU]) + ay * (v * sy[IR] + r * sy[IV]));
  h[IU] = u - (ax * (u * sx[IU] + sx[IP] / r) + ay * (v * sy[IU]));
  h[IV] = v - (ax * (u * sx[IV]) + ay * (v * sy[IV] + sy[IP] / r));
  h[IP] = pr - (ax * (gamma0 * pr * sx[IU] + u * sx[IP]) + ay * (gamma0 * pr * sy[IV] + v * sy[IP]));
  return h;
}

// ---------------------------------------------------------------- BoundaryConditions.h
// BoundaryConditions.h:13-16, 18-46, 48-71 and the two passes of 82-147.
void fillBoundaries(fv2d_oracle *o, std::vector<real_t> &Q) {
  const Grid &g = o->g;
  const int bcx = o->p.boundary_x, bcy = o->p.boundary_y;
  // X pass over range_xbound = [0, Ng) x [jbeg, jend) (SimInfo.h:560)
#pragma omp parallel for schedule(static)
  for (int j = g.jbeg; j < g.jend; ++j) {
    for (int i = 0; i < g.Ng; ++i) {
      auto fill = [&](int ig, int iref) -> State {
        switch (bcx) {
          case FV2D_BC_REFLECTING: {
            int ipiv = (ig < iref ? g.ibeg : g.iend);
            int isym = 2 * ipiv - ig - 1;
            State q = o->get(Q, isym, j);
            q[IU] *= -1.0;
            return q;
          }
          case FV2D_BC_PERIODIC: {
            int is = (ig < g.ibeg) ? ig + g.Nx : ig - g.Nx;
            return o->get(Q, is, j);
          }
          default:
            return o->get(Q, iref, j);
        }
      };
      const int ileft = i, iright = g.iend + i;
      o->set(Q, ileft, j, fill(ileft, g.ibeg));
      o->set(Q, iright, j, fill(iright, g.iend - 1));
    }
  }
  // Y pass over range_ybound = [0, Ntx) x [0, Ng) (SimInfo.h:561)
#pragma omp parallel for schedule(static)
  for (int j = 0; j < g.Ng; ++j) {
    for (int i = 0; i < g.Ntx; ++i) {
      auto fill = [&](int jg, int jref) -> State {
        switch (bcy) {
          case FV2D_BC_REFLECTING: {
            int jpiv = (jg < jref ? g.jbeg : g.jend);
            int jsym = 2 * jpiv - jg - 1;
            State q = o->get(Q, i, jsym);
            q[IV] *= -1.0;
            return q;
          }
          case FV2D_BC_PERIODIC: {
            int js = (jg < g.jbeg) ? jg + g.Ny : jg - g.Ny;
            return o->get(Q, i, js);
          }
          default:
            return o->get(Q, i, jref);
        }
      };
      const int jtop = j, jbot = g.jend + j;
      o->set(Q, i, jtop, fill(jtop, g.jbeg));
      o->set(Q, i, jbot, fill(jbot, g.jend - 1));
    }
  }
}

// ---------------------------------------------------------------- Update.h
// Update.h:59-91 over range_slopes = [ibeg-1, iend+1) x [jbeg-1, jend+1)
void computeSlopes(fv2d_oracle *o) {
  const Grid &g = o->g;
  const auto &Q = o->Q;
  auto minmod = [](real_t dL, real_t dR) -> real_t {
    if (dL * dR < 0.0) return 0.0;
    if (std::fabs(dL) < std::fabs(dR)) return dL;
    return dR;
  };
#pragma omp parallel for schedule(static)
  for (int j = g.jbeg - 1; j < g.jend + 1; ++j)
    for (int i = g.ibeg - 1; i < g.iend + 1; ++i)
      for (int v = 0; v < 4; ++v) {
        real_t dL = Q[o->at(j, i, v)] - Q[o->at(j, i - 1, v)];
        real_t dR = Q[o->at(j, i + 1, v)] - Q[o->at(j, i, v)];
        real_t dU = Q[o->at(j, i, v)] - Q[o->at(j - 1, i, v)];
        real_t dD = Q[o->at(j + 1, i, v)] - Q[o->at(j, i, v)];
        o->slopesX[o->at(j, i, v)] = minmod(dL, dR);
        o->slopesY[o->at(j, i, v)] = minmod(dU, dD);
      }
}

// Update.h:15-37.  PCM_WB computes a pressure correction and then falls
// through to the PCM branch, so its result is the PCM state.  The
// MUSCL-Hancock extension evaluates the half-step state first.
State reconstruct(const fv2d_oracle *o, const std::vector<real_t> &slopes, int i, int j, real_t sign, Dir d,
                  real_t dt) {
  State q = o->get(o->Q, i, j);
  State slope = o->get(slopes, i, j);
  State res;
  switch (o->p.reconstruction) {
    case FV2D_PLM:
      res = q + slope * sign * 0.5;
      break;
    case FV2D_MUSCL_HANCOCK: {
      const real_t ax = 0.5 * dt / o->g.dx, ay = 0.5 * dt / o->g.dy;
      State qh = hancock(q, o->get(o->slopesX, i, j), o->get(o->slopesY, i, j), ax, ay, o->p.gamma0);
      res = qh + slope * sign * 0.5;
      break;
    }
    default:
      res = q;
      break;
  }
  return swap_component(res, d);
}

// Update.h:93-174
void computeFluxesAndUpdate(fv2d_oracle *o, std::vector<real_t> &Unew, real_t dt) {
  const Grid &g = o->g;
  const fv2d_params &p = o->p;
  const auto &Q = o->Q;
#pragma omp parallel for schedule(static)
  for (int j = g.jbeg; j < g.jend; ++j)
    for (int i = g.ibeg; i < g.iend; ++i) {
      auto updateAlongDir = [&](Dir d) {
        const auto &slopes = (d == IX ? o->slopesX : o->slopesY);
        int dxm = (d == IX ? -1 : 0), dxp = (d == IX ? 1 : 0);
        int dym = (d == IY ? -1 : 0), dyp = (d == IY ? 1 : 0);
        State qCL = reconstruct(o, slopes, i, j, -1.0, d, dt);
        State qCR = reconstruct(o, slopes, i, j, 1.0, d, dt);
        State qL = reconstruct(o, slopes, i + dxm, j + dym, 1.0, d, dt);
        State qR = reconstruct(o, slopes, i + dxp, j + dyp, -1.0, d, dt);
        const real_t gdx = (d == IX ? p.gx * g.dx : p.gy * g.dy);
        auto riemann = [&](const State &a, const State &b, State &flux, real_t &pout) {
          switch (p.riemann_solver) {
            case FV2D_HLL: hll(a, b, flux, pout, p); break;
            case FV2D_FSLP: fslp(a, b, flux, pout, gdx, p); break;
            default: hllc(a, b, flux, pout, p); break;
          }
        };
        State fluxL, fluxR;
        real_t poutL, poutR;
        riemann(qL, qCL, fluxL, poutL);
        riemann(qCR, qR, fluxR, poutR);
        fluxL = swap_component(fluxL, d);
        fluxR = swap_component(fluxR, d);
        if (p.well_balanced_flux_at_y_bc && (j == g.jbeg || j == g.jend - 1) && d == IY) {
          real_t gv = getGravity(g, p, i, j, d);
          if (j == g.jbeg)
            fluxL = State{{0.0, 0.0, poutR - Q[o->at(j, i, IR)] * gv * g.dy, 0.0}};
          else
            fluxR = State{{0.0, 0.0, poutL + Q[o->at(j, i, IR)] * gv * g.dy, 0.0}};
        }
        State un = o->get(Unew, i, j);
        un += dt * (fluxL - fluxR) / (d == IX ? g.dx : g.dy);
        if (p.gravity_mode != FV2D_GRAV_NONE) {
          real_t gv = getGravity(g, p, i, j, d);
          un[IV] += dt * Q[o->at(j, i, IR)] * gv;
          un[IE] += dt * 0.5 * (fluxL[IR] + fluxR[IR]) * gv;
        }
        o->set(Unew, i, j, un);
      };
      updateAlongDir(IX);
      updateAlongDir(IY);
    }
}

// ThermalConduction.h:36-108
void applyThermalConduction(fv2d_oracle *o, std::vector<real_t> &Unew, real_t dt) {
  const Grid &g = o->g;
  const fv2d_params &p = o->p;
  const auto &Q = o->Q;
  const real_t dx = g.dx, dy = g.dy;
#pragma omp parallel for schedule(static)
  for (int j = g.jbeg; j < g.jend; ++j)
    for (int i = g.ibeg; i < g.iend; ++i) {
      real_t x = posX(g, i), y = posY(g, j);
      real_t kC = computeKappa(g, p, i, j);
      real_t kappaL = 0.5 * (kC + computeKappa(g, p, (int)(x - dx), (int)y));
      real_t kappaR = 0.5 * (kC + computeKappa(g, p, (int)(x + dx), (int)y));
      real_t kappaU = 0.5 * (kC + computeKappa(g, p, (int)x, (int)(y - dy)));
      real_t kappaD = 0.5 * (kC + computeKappa(g, p, (int)x, (int)(y + dy)));
      real_t TC = Q[o->at(j, i, IP)] / Q[o->at(j, i, IR)];
      real_t TL = Q[o->at(j, i - 1, IP)] / Q[o->at(j, i - 1, IR)];
      real_t TR = Q[o->at(j, i + 1, IP)] / Q[o->at(j, i + 1, IR)];
      real_t TU = Q[o->at(j - 1, i, IP)] / Q[o->at(j - 1, i, IR)];
      real_t TD = Q[o->at(j + 1, i, IP)] / Q[o->at(j + 1, i, IR)];
      real_t FL = kappaL * (TC - TL) / dx;
      real_t FR = kappaR * (TR - TC) / dx;
      real_t FU = kappaU * (TC - TU) / dy;
      real_t FD = kappaD * (TD - TC) / dy;
      if (j == g.jbeg && p.bctc_ymin != FV2D_BCTC_NONE) {
        if (p.bctc_ymin == FV2D_BCTC_FIXED_TEMPERATURE)
          FL = kappaL * 2.0 * (TC - p.bctc_ymin_value) / dy;
        else if (p.bctc_ymin == FV2D_BCTC_FIXED_GRADIENT)
          FL = kappaL * p.bctc_ymin_value;
      }
      if (j == g.jend - 1 && p.bctc_ymax != FV2D_BCTC_NONE) {
        if (p.bctc_ymax == FV2D_BCTC_FIXED_TEMPERATURE)
          FR = kappaR * 2.0 * (p.bctc_ymax_value - TC) / dy;
        else if (p.bctc_ymax == FV2D_BCTC_FIXED_GRADIENT)
          FR = kappaR * p.bctc_ymax_value;
      }
      Unew[o->at(j, i, IE)] += dt / dx * (FR - FL) + dt / dy * (FD - FU);
    }
}

// Viscosity.h:27-119
void applyViscosity(fv2d_oracle *o, std::vector<real_t> &Unew, real_t dt) {
  const Grid &g = o->g;
  const fv2d_params &p = o->p;
  const real_t dx = g.dx, dy = g.dy;
#pragma omp parallel for schedule(static)
  for (int j = g.jbeg; j < g.jend; ++j)
    for (int i = g.ibeg; i < g.iend; ++i) {
      State st[3][3];
      constexpr real_t four_thirds = 4.0 / 3.0;
      constexpr real_t two_thirds = 2.0 / 3.0;
      for (int di = -1; di < 2; ++di)
        for (int dj = -1; dj < 2; ++dj) st[dj + 1][di + 1] = o->get(o->Q, i + di, j + dj);
      auto viscousFlux = [&](Dir d) {
        State flux{{0.0, 0.0, 0.0, 0.0}};
        const real_t one_over_dx = 1.0 / dx;
        const real_t one_over_dy = 1.0 / dy;
        real_t mu = computeMu(p);
        for (int side = 1; side < 3; ++side) {
          real_t sign = (side == 1 ? -1.0 : 1.0);
          if (d == IX) {
            State qi = 0.5 * (st[1][side] + st[1][side - 1]);
            real_t dudx = one_over_dx * (st[1][side][IU] - st[1][side - 1][IU]);
            real_t dvdx = one_over_dx * (st[1][side][IV] - st[1][side - 1][IV]);
            real_t dudy = 0.25 * one_over_dy *
                          (st[2][side][IU] - st[0][side][IU] + st[2][side - 1][IU] - st[0][side - 1][IU]);
            real_t dvdy = 0.25 * one_over_dy *
                          (st[2][side][IV] - st[0][side][IV] + st[2][side - 1][IV] - st[0][side - 1][IV]);
            const real_t tau_xx = four_thirds * dudx - two_thirds * dvdy;
            const real_t tau_xy = dvdx + dudy;
            flux[IU] += sign * mu * tau_xx;
            flux[IV] += sign * mu * tau_xy;
            flux[IE] += sign * mu * (tau_xx * qi[IU] + tau_xy * qi[IV]);
          } else {
            State qi = 0.5 * (st[side][1] + st[side - 1][1]);
            real_t dudy = one_over_dy * (st[side][1][IU] - st[side - 1][1][IU]);
            real_t dvdy = one_over_dy * (st[side][1][IV] - st[side - 1][1][IV]);
            real_t dudx = 0.25 * one_over_dx *
                          (st[side][2][IU] - st[side][0][IU] + st[side - 1][2][IU] - st[side - 1][0][IU]);
            real_t dvdx = 0.25 * one_over_dx *
                          (st[side][2][IV] - st[side][0][IV] + st[side - 1][2][IV] - st[side - 1][0][IV]);
            const real_t tau_yy = four_thirds * dvdy - two_thirds * dudx;
            const real_t tau_xy = dvdx + dudy;
            flux[IU] += sign * mu * tau_xy;
            flux[IV] += sign * mu * tau_yy;
            flux[IE] += sign * mu * (tau_xy * qi[IU] + tau_yy * qi[IV]);
          }
        }
        return flux;
      };
      State vf_x = viscousFlux(IX);
      State vf_y = viscousFlux(IY);
      State un = o->get(Unew, i, j);
      un += dt * (vf_x + vf_y);
      o->set(Unew, i, j, un);
    }
}

// Update.h:176-191
void eulerStep(fv2d_oracle *o, std::vector<real_t> &Unew, real_t dt) {
  fillBoundaries(o, o->Q);
  if (o->p.reconstruction == FV2D_PLM || o->p.reconstruction == FV2D_MUSCL_HANCOCK) computeSlopes(o);
  computeFluxesAndUpdate(o, Unew, dt);
  if (o->p.thermal_conductivity_active) applyThermalConduction(o, Unew, dt);
  if (o->p.viscosity_active) applyViscosity(o, Unew, dt);
}

// SimInfo.h:576-587 over range_tot
void consToPrimGrid(fv2d_oracle *o, const std::vector<real_t> &U) {
  const Grid &g = o->g;
#pragma omp parallel for schedule(static)
  for (int j = 0; j < g.Nty; ++j)
    for (int i = 0; i < g.Ntx; ++i) o->set(o->Q, i, j, consToPrim(o->get(U, i, j), o->p));
}

// SimInfo.h:589-600 over range_tot
void primToConsGrid(fv2d_oracle *o) {
  const Grid &g = o->g;
#pragma omp parallel for schedule(static)
  for (int j = 0; j < g.Nty; ++j)
    for (int i = 0; i < g.Ntx; ++i) o->set(o->U, i, j, primToCons(o->get(o->Q, i, j), o->p));
}

// Update.h:193-222
void update(fv2d_oracle *o, real_t dt) {
  if (o->p.time_stepping == FV2D_TS_EULER) {
    eulerStep(o, o->U, dt);
    return;
  }
  const Grid &g = o->g;
  o->U0 = o->U;
  o->Ustar = o->U;
  eulerStep(o, o->Ustar, dt);
  o->U = o->Ustar;
  consToPrimGrid(o, o->Ustar);
  eulerStep(o, o->U, dt);
#pragma omp parallel for schedule(static)
  for (int j = g.jbeg; j < g.jend; ++j)
    for (int i = g.ibeg; i < g.iend; ++i)
      for (int v = 0; v < 4; ++v) o->U[o->at(j, i, v)] = 0.5 * (o->U0[o->at(j, i, v)] + o->U[o->at(j, i, v)]);
}

// SimInfo.h:602-636 over range_dom
void checkNegatives(fv2d_oracle *o) {
  const Grid &g = o->g;
  const real_t eps = o->p.epsilon_reset_negative;
  uint64_t nd = 0, np = 0, nn = 0;
#pragma omp parallel for schedule(static) reduction(+ : nd, np, nn)
  for (int j = g.jbeg; j < g.jend; ++j)
    for (int i = g.ibeg; i < g.iend; ++i) {
      real_t *q = &o->Q[o->at(j, i, 0)];
      if (q[IR] < 0) {
        q[IR] = eps;
        nd++;
      }
      if (q[IP] < 0) {
        q[IP] = eps;
        np++;
      }
      for (int v = 0; v < 4; ++v)
        if (std::isnan(q[v])) nn++;
    }
  o->counters[0] = nd;
  o->counters[1] = np;
  o->counters[2] = nn;
}

// ComputeDt.h:18-65 (max reductions with the fmax semantics of :421-423)
void computeDt(const fv2d_oracle *o, real_t out[4]) {
  const Grid &g = o->g;
  const fv2d_params &p = o->p;
  real_t hyp, tc, visc;
  int nt = 1;
#ifdef _OPENMP
  nt = omp_get_max_threads();
#endif
  // Kokkos::Max starts every partial result from the lowest double.
  const real_t lowest = -std::numeric_limits<real_t>::max();
  std::vector<real_t> ph(nt, lowest), pt(nt, lowest), pv(nt, lowest);
#pragma omp parallel
  {
    int tid = 0;
#ifdef _OPENMP
    tid = omp_get_thread_num();
#endif
    real_t lh = lowest, lt = lowest, lv = lowest;
#pragma omp for schedule(static)
    for (int j = g.jbeg; j < g.jend; ++j)
      for (int i = g.ibeg; i < g.iend; ++i) {
        State q = o->get(o->Q, i, j);
        real_t cs = speedOfSound(q, p);
        real_t h = (cs + std::fabs(q[IU])) / g.dx + (cs + std::fabs(q[IV])) / g.dy;
        real_t t = p.epsilon;
        if (p.thermal_conductivity_active)
          t = std::fmax(2.0 * computeKappa(g, p, i, j) / (g.dx * g.dx), 2.0 * computeKappa(g, p, i, j) / (g.dy * g.dy));
        real_t v = p.epsilon;
        if (p.viscosity_active) v = std::fmax(2.0 * computeMu(p) / (g.dx * g.dx), 2.0 * computeMu(p) / (g.dy * g.dy));
        lh = std::fmax(lh, h);
        lt = std::fmax(lt, t);
        lv = std::fmax(lv, v);
      }
    ph[tid] = lh;
    pt[tid] = lt;
    pv[tid] = lv;
  }
  hyp = ph[0];
  tc = pt[0];
  visc = pv[0];
  for (int k = 1; k < nt; ++k) {
    hyp = std::fmax(hyp, ph[k]);
    tc = std::fmax(tc, pt[k]);
    visc = std::fmax(visc, pv[k]);
  }
  out[0] = p.CFL / std::max({hyp, tc, visc});
  out[1] = hyp;
  out[2] = tc;
  out[3] = visc;
}

// ---------------------------------------------------------------- Init.h
uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

void initCell(const fv2d_oracle *o, int problem, int i, int j, real_t *q) {
  const Grid &g = o->g;
  const fv2d_params &p = o->p;
  const real_t x = posX(g, i), y = posY(g, j);
  const real_t xmid = 0.5 * (g.xmin + g.xmax), ymid = 0.5 * (g.ymin + g.ymax);
  const int64_t cell = (int64_t)(j - g.jbeg) * g.Nx + (i - g.ibeg);
  switch (problem) {
    case FV2D_PB_SOD_X:  // Init.h:20-35 (states parameterised; defaults are the reference's)
    case FV2D_PB_SOD_Y:  // Init.h:83-98
    {
      real_t c = (problem == FV2D_PB_SOD_X) ? x : y;
      if (c <= 0.5) {
        q[IR] = p.sod_rho_left;
        q[IP] = p.sod_p_left;
        q[IU] = 0.0;
      } else {
        q[IR] = p.sod_rho_right;
        q[IP] = p.sod_p_right;
        q[IU] = 0.0;
      }
      break;
    }
    case FV2D_PB_GRESHO_VORTEX: {  // Init.h:42-78
      const real_t xr = x - xmid, yr = y - ymid;
      const real_t r = std::sqrt(xr * xr + yr * yr);
      const real_t p0 = p.gresho_density / (p.gamma0 * p.gresho_Mach * p.gresho_Mach);
      q[IR] = p.gresho_density;
      real_t u_phi;
      if (r < 0.2) {
        u_phi = 5.0 * r;
        q[IP] = p0 + 12.5 * r * r;
      } else if (r < 0.4) {
        u_phi = 2.0 - 5.0 * r;
        q[IP] = p0 + 12.5 * r * r + 4.0 * (1.0 - 5.0 * r + std::log(5.0 * r));
      } else {
        u_phi = 0.0;
        q[IP] = p0 - 2.0 + 4.0 * std::log(2.0);
      }
      const real_t xnr = xr / r, ynr = yr / r;
      q[IU] = -ynr * u_phi;
      q[IV] = xnr * u_phi;
      break;
    }
    case FV2D_PB_BLAST: {  // Init.h:103-131
      real_t xr = xmid - x, yr = ymid - y;
      real_t r = std::sqrt(xr * xr + yr * yr);
      if (r < 0.2) {
        q[IR] = 1.0; q[IU] = 0.0; q[IV] = 0.0; q[IP] = 10.0;
      } else {
        q[IR] = 1.2; q[IU] = 0.0; q[IV] = 0.0; q[IP] = 0.1;
      }
      break;
    }
    case FV2D_PB_H84: {  // Init.h:136-154 (Kokkos XorShift pool replaced by the counter-based generator)
      real_t rho = std::pow(y, p.m1);
      real_t prs = std::pow(y, p.m1 + 1.0);
      real_t pert = p.h84_pert * (-0.5 + fv2d_oracle_uniform(p.seed, cell, 0));
      q[IR] = rho; q[IU] = 0.0; q[IV] = pert; q[IP] = prs;
      break;
    }
    case FV2D_PB_C91: {  // Init.h:159-180
      real_t T = (1.0 + p.theta1 * y);
      real_t rho = std::pow(T, p.m1);
      real_t prs = std::pow(T, p.m1 + 1.0);
      real_t pert = p.c91_pert * (-0.5 + fv2d_oracle_uniform(p.seed, cell, 0));
      prs = prs * (1.0 + pert);
      q[IR] = rho; q[IU] = 0.0; q[IV] = 0.0; q[IP] = prs;
      break;
    }
    case FV2D_PB_DIFFUSION: {  // Init.h:185-206
      real_t x0 = (x - xmid), y0 = (y - ymid);
      real_t r = std::sqrt(x0 * x0 + y0 * y0);
      q[IR] = (r < 0.2) ? 1.0 : 0.1;
      q[IP] = 1.0; q[IU] = 1.0; q[IV] = 1.0;
      break;
    }
    case FV2D_PB_RAYLEIGH_TAYLOR: {  // Init.h:211-237
      const real_t P0 = 2.5;
      if (y < ymid) {
        q[IR] = 1.0; q[IU] = 0.0; q[IP] = P0 + 0.1 * p.gy * y;
      } else {
        q[IR] = 2.0; q[IU] = 0.0; q[IP] = P0 + 0.1 * p.gy * y;
      }
      if (y > -1.0 / 3.0 && y < 1.0 / 3.0)
        q[IV] = 0.01 * (1.0 + std::cos(4 * M_PI * x)) * (1 + std::cos(3.0 * M_PI * y)) / 4.0;
      break;
    }
    case FV2D_PB_KELVIN_HELMHOLTZ: {  // Init.h:245-265
      const real_t q1 = std::tanh((y - p.kh_y1) / p.kh_a);
      const real_t q2 = std::tanh((y - p.kh_y2) / p.kh_a);
      const real_t s2 = p.kh_sigma * p.kh_sigma;
      const real_t dy1 = (y - p.kh_y1) * (y - p.kh_y1);
      const real_t dy2 = (y - p.kh_y2) * (y - p.kh_y2);
      q[IR] = 1.0 + p.kh_rho_fac * 0.5 * (q1 - q2);
      q[IU] = p.kh_uflow * (q1 - q2 - 1.0);
      q[IV] = p.kh_amp * std::sin(2.0 * M_PI * x) * (std::exp(-dy1 / s2) + std::exp(-dy2 / s2));
      q[IP] = p.kh_P0;
      break;
    }
    case FV2D_PB_SEDOV: {  // extension: point energy E0 spread over the cells within r0
      const real_t xr = x - xmid, yr = y - ymid;
      const real_t r = std::sqrt(xr * xr + yr * yr);
      q[IR] = p.sedov_rho; q[IU] = 0.0; q[IV] = 0.0;
      q[IP] = (r <= p.sedov_r0) ? (p.gamma0 - 1.0) * p.sedov_E0 / (M_PI * p.sedov_r0 * p.sedov_r0) : p.sedov_p_ambient;
      break;
    }
    case FV2D_PB_KH_STEP: {  // extension: sharp shear layer + sin(4 pi x) + seeded noise
      const bool in = std::fabs(y - ymid) < 0.25;
      q[IR] = in ? p.khs_rho_in : p.khs_rho_out;
      q[IU] = (in ? p.khs_u : -p.khs_u) + p.khs_noise * (2.0 * fv2d_oracle_uniform(p.seed, cell, 1) - 1.0);
      q[IV] = p.khs_amp * std::sin(4.0 * M_PI * x) + p.khs_noise * (2.0 * fv2d_oracle_uniform(p.seed, cell, 2) - 1.0);
      q[IP] = p.khs_p0;
      break;
    }
    case FV2D_PB_RT_HYDROSTATIC: {  // extension: hydrostatic two-layer column under constant gy
      const real_t rho = (y > p.rt_y_interface) ? p.rt_rho_top : p.rt_rho_bottom;
      q[IR] = rho;
      q[IU] = 0.0;
      q[IV] = p.rt_amp * (1.0 + std::cos(4.0 * M_PI * x)) * (1.0 + std::cos(3.0 * M_PI * (y - p.rt_y_interface))) / 4.0;
      q[IP] = p.rt_p_interface + rho * p.gy * (y - p.rt_y_interface);
      break;
    }
    default:
      break;
  }
}

bool validProblem(int pb) {
  return (pb >= FV2D_PB_SOD_X && pb <= FV2D_PB_GRESHO_VORTEX) || pb == FV2D_PB_SEDOV || pb == FV2D_PB_KH_STEP ||
         pb == FV2D_PB_RT_HYDROSTATIC;
}

}  // namespace

extern "C" {

double fv2d_oracle_uniform(int32_t seed, int64_t cell, int32_t stream) {
  uint64_t key = ((uint64_t)(uint32_t)seed << 32) ^ ((uint64_t)cell * 4u + (uint64_t)(uint32_t)stream);
  return (double)(mix64(key) >> 11) * 0x1.0p-53;
}

void fv2d_oracle_params_default(fv2d_params *p) {
  std::memset(p, 0, sizeof(*p));
  p->struct_size = sizeof(fv2d_params);
  p->Nx = 32; p->Ny = 32; p->Nghosts = 2;
  p->xmin = 0.0; p->xmax = 1.0; p->ymin = 0.0; p->ymax = 1.0;
  p->CFL = 0.8;
  p->boundary_x = FV2D_BC_REFLECTING; p->boundary_y = FV2D_BC_REFLECTING;
  p->reconstruction = FV2D_PCM;
  p->riemann_solver = FV2D_HLLC;
  p->time_stepping = FV2D_TS_EULER;
  p->tend = 1.0; p->save_freq = 1.0e-1;
  p->gamma0 = 5.0 / 3.0;
  p->epsilon = 1.0e-6;
  p->epsilon_reset_negative = 1.0e-8;
  p->well_balanced_flux_at_y_bc = 0;
  p->fslp_K = 1.1;
  p->seed = 12345;
  p->log_frequency = 10;
  p->gravity_mode = FV2D_GRAV_NONE;
  p->analytical_gravity_mode = FV2D_AGM_HOT_BUBBLE;
  p->gx = 0.0; p->gy = 0.0; p->hot_bubble_g0 = 0.0;
  p->thermal_conductivity_active = 0;
  p->thermal_conductivity_mode = FV2D_TCM_CONSTANT;
  p->kappa = 0.0;
  p->bctc_ymin = FV2D_BCTC_NONE; p->bctc_ymax = FV2D_BCTC_NONE;
  p->bctc_ymin_value = 1.0; p->bctc_ymax_value = 1.0;
  p->viscosity_active = 0; p->viscosity_mode = FV2D_VSC_CONSTANT; p->mu = 0.0;
  p->m1 = 1.0; p->theta1 = 10.0; p->m2 = 1.0; p->theta2 = 10.0;
  p->h84_pert = 1.0e-4; p->c91_pert = 1.0e-3;
  p->kh_a = 0.05; p->kh_amp = 0.01; p->kh_P0 = 1.0; p->kh_rho_fac = 0.0; p->kh_sigma = 0.2;
  p->kh_uflow = 1.0; p->kh_y1 = 0.5; p->kh_y2 = 1.5;
  p->gresho_density = 1.0; p->gresho_Mach = 0.1;
  p->sod_rho_left = 1.0; p->sod_p_left = 1.0; p->sod_rho_right = 0.125; p->sod_p_right = 0.1;
  p->sedov_E0 = 1.0; p->sedov_r0 = 0.02; p->sedov_p_ambient = 1.0e-5; p->sedov_rho = 1.0;
  p->khs_rho_in = 2.0; p->khs_rho_out = 1.0; p->khs_u = 0.5; p->khs_p0 = 2.5; p->khs_amp = 0.01; p->khs_noise = 1.0e-3;
  p->rt_rho_top = 2.0; p->rt_rho_bottom = 1.0; p->rt_p_interface = 2.5; p->rt_y_interface = 0.75; p->rt_amp = 0.01;
}

int fv2d_oracle_create(const fv2d_params *p, fv2d_oracle **out) {
  if (!p || !out || p->struct_size != sizeof(fv2d_params)) return FV2D_ERR_INVALID;
  if (p->Nx < 2 || p->Ny < 2 || p->Nghosts < 2) return FV2D_ERR_INVALID;
  fv2d_oracle *o = new (std::nothrow) fv2d_oracle();
  if (!o) return FV2D_ERR_NOMEM;
  o->p = *p;
  Grid &g = o->g;
  g.Nx = p->Nx; g.Ny = p->Ny; g.Ng = p->Nghosts;
  g.Ntx = g.Nx + 2 * g.Ng; g.Nty = g.Ny + 2 * g.Ng;
  g.ibeg = g.Ng; g.iend = g.Ng + g.Nx; g.jbeg = g.Ng; g.jend = g.Ng + g.Ny;
  g.xmin = p->xmin; g.xmax = p->xmax; g.ymin = p->ymin; g.ymax = p->ymax;
  g.dx = (g.xmax - g.xmin) / g.Nx;  // SimInfo.h:375-376
  g.dy = (g.ymax - g.ymin) / g.Ny;
  size_t n = (size_t)g.Ntx * g.Nty * 4;
  try {
    o->Q.assign(n, 0.0);
    o->U.assign(n, 0.0);
    o->slopesX.assign(n, 0.0);
    o->slopesY.assign(n, 0.0);
  } catch (...) {
    delete o;
    return FV2D_ERR_NOMEM;
  }
  *out = o;
  return FV2D_OK;
}

void fv2d_oracle_destroy(fv2d_oracle *o) { delete o; }

int fv2d_oracle_init_problem(fv2d_oracle *o, int problem) {
  if (!o || !validProblem(problem)) return FV2D_ERR_INVALID;
  const Grid &g = o->g;
  std::fill(o->Q.begin(), o->Q.end(), 0.0);  // Kokkos views start zeroed (main.cpp:33-34)
#pragma omp parallel for schedule(static)
  for (int j = g.jbeg; j < g.jend; ++j)
    for (int i = g.ibeg; i < g.iend; ++i) initCell(o, problem, i, j, &o->Q[o->at(j, i, 0)]);
  fillBoundaries(o, o->Q);
  primToConsGrid(o);
  return FV2D_OK;
}

int fv2d_oracle_set_prim(fv2d_oracle *o, const double *q) {
  if (!o || !q) return FV2D_ERR_INVALID;
  const Grid &g = o->g;
  for (int j = 0; j < g.Ny; ++j)
    std::memcpy(&o->Q[o->at(j + g.jbeg, g.ibeg, 0)], q + (size_t)j * g.Nx * 4, sizeof(double) * 4 * g.Nx);
  fillBoundaries(o, o->Q);
  primToConsGrid(o);
  return FV2D_OK;
}

int fv2d_oracle_get_prim(const fv2d_oracle *o, double *q) {
  if (!o || !q) return FV2D_ERR_INVALID;
  const Grid &g = o->g;
  for (int j = 0; j < g.Ny; ++j)
    std::memcpy(q + (size_t)j * g.Nx * 4, &o->Q[o->at(j + g.jbeg, g.ibeg, 0)], sizeof(double) * 4 * g.Nx);
  return FV2D_OK;
}

int fv2d_oracle_get_cons(const fv2d_oracle *o, double *u) {
  if (!o || !u) return FV2D_ERR_INVALID;
  const Grid &g = o->g;
  for (int j = 0; j < g.Ny; ++j)
    std::memcpy(u + (size_t)j * g.Nx * 4, &o->U[o->at(j + g.jbeg, g.ibeg, 0)], sizeof(double) * 4 * g.Nx);
  return FV2D_OK;
}

int fv2d_oracle_compute_dt(const fv2d_oracle *o, double out[4]) {
  if (!o || !out) return FV2D_ERR_INVALID;
  computeDt(o, out);
  return FV2D_OK;
}

int fv2d_oracle_update(fv2d_oracle *o, double dt) {
  if (!o) return FV2D_ERR_INVALID;
  update(o, dt);
  consToPrimGrid(o, o->U);
  checkNegatives(o);
  return FV2D_OK;
}

int fv2d_oracle_round_cons_f32(fv2d_oracle *o, const double *bg) {
  if (!o) return FV2D_ERR_INVALID;
  const Grid &g = o->g;
  const double zero[4] = {0.0, 0.0, 0.0, 0.0};
  const double *b = bg ? bg : zero;
#pragma omp parallel for schedule(static)
  for (int j = 0; j < g.Nty; ++j)
    for (int i = 0; i < g.Ntx; ++i)
      for (int v = 0; v < 4; ++v) {
        double &x = o->U[o->at(j, i, v)];
        x = (double)(float)(x - b[v]) + b[v];
      }
  consToPrimGrid(o, o->U);
  checkNegatives(o);
  return FV2D_OK;
}

int fv2d_oracle_get_counters(const fv2d_oracle *o, uint64_t out[3]) {
  if (!o || !out) return FV2D_ERR_INVALID;
  for (int k = 0; k < 3; ++k) out[k] = o->counters[k];
  return FV2D_OK;
}

int fv2d_oracle_run(fv2d_oracle *o, double tend, int max_steps, double *t_io, int *nsteps, double *dts) {
  if (!o || !t_io || !nsteps) return FV2D_ERR_INVALID;
  double t = *t_io;
  int n = 0;
  while (t + o->p.epsilon < tend && n < max_steps) {  // main.cpp:62-84
    double d[4];
    computeDt(o, d);
    if (dts) dts[n] = d[0];
    fv2d_oracle_update(o, d[0]);
    t += d[0];
    ++n;
  }
  *t_io = t;
  *nsteps = n;
  return FV2D_OK;
}

void fv2d_oracle_set_threads(int n) {
  g_threads = n;
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#endif
}

int fv2d_oracle_get_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // extern "C"
