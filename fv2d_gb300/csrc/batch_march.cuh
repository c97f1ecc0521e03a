// batch_march.cuh -- register-resident FP32 step of the batched service.
//
// One warp owns a work item: a strip of 32 padded columns (28 interior
// columns plus a 2-column halo on each side) of one simulation, over a band
// of rows (its height is the simulation's `band`, which the service sets per
// lane).  Lane l holds column i0 + l and marches down the band: each new
// row is loaded once (coalesced), converted to primitives and kept in a
// 4-row register window; x neighbours come from warp shuffles, y neighbours
// from the window.  Every face is solved once (x faces in the lane on their
// right, y faces as the march crosses them), so the step needs no shared
// memory, no barriers and little index arithmetic.  Same physics and update
// order as the reference (States.h:32-43, RiemannSolvers.h:7-171,
// Update.h:93-174, ThermalConduction.h:36-108, Viscosity.h:27-119), and the
// same per-simulation commit of the step (ComputeDt.h:64, main.cpp:62-83).
//
// Two kernels of item bodies, each compiled per Riemann solver and
// reconstruction so that the row loop carries neither branch:
//   - batch_march_kernel, for the plain and the diffusive families: HLL or
//     HLLC, PCM or PLM, constant gravity, constant conductivity, viscosity;
//   - batch_march_ext_kernel, for the extended family: also FSLP and the
//     MUSCL-Hancock predictor, gravity and conductivity from per-row tables
//     (analytical gravity, B02 conductivity), the y-boundary conduction
//     modes and the well-balanced y-boundary flux.
// Both take SSP-RK2 as two launches (stage_buffers) and store the state as
// offsets from the simulation's background density and energy.
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
// Component-wise operations on the state's two halves (rho, u) and (v, p) as
// packed binary32 pairs (sm_100 FADD2 / FMUL2 / FFMA2): one issue per pair,
// the same single rounding per component as the scalar forms.
__device__ __forceinline__ float2 lo2(const S4<float> &a) { return make_float2(a.r, a.u); }
__device__ __forceinline__ float2 hi2(const S4<float> &a) { return make_float2(a.v, a.p); }
__device__ __forceinline__ S4<float> join4(float2 lo, float2 hi) { return S4<float>{lo.x, lo.y, hi.x, hi.y}; }
__device__ __forceinline__ S4<float> sub4(const S4<float> &a, const S4<float> &b) {
  const float2 m1 = make_float2(-1.f, -1.f);
  return join4(__ffma2_rn(lo2(b), m1, lo2(a)), __ffma2_rn(hi2(b), m1, hi2(a)));
}
// minmod slope from the differences to the left and right neighbours
// (Update.h:59-91); each difference is formed once and serves the slopes of
// both cells it separates
__device__ __forceinline__ float minmod_p(float dl, float dr, float prod) {
  const float m = fabsf(dl) < fabsf(dr) ? dl : dr;
  return prod < 0.f ? 0.f : m;
}
__device__ __forceinline__ S4<float> slope4(const S4<float> &dl, const S4<float> &dr) {
  const float2 pl = __fmul2_rn(lo2(dl), lo2(dr)), ph = __fmul2_rn(hi2(dl), hi2(dr));
  return S4<float>{minmod_p(dl.r, dr.r, pl.x), minmod_p(dl.u, dr.u, pl.y), minmod_p(dl.v, dr.v, ph.x),
                   minmod_p(dl.p, dr.p, ph.y)};
}
// reconstructed face state q + slope * sign * 0.5 (Update.h:25), one
// multiply-add per field
__device__ __forceinline__ S4<float> face4(const S4<float> &q, const S4<float> &s, float half) {
  const float2 h = make_float2(half, half);
  return join4(__ffma2_rn(h, lo2(s), lo2(q)), __ffma2_rn(h, hi2(s), hi2(q)));
}
__device__ __forceinline__ S4<float> swap_uv(const S4<float> &q) { return S4<float>{q.r, q.v, q.u, q.p}; }

// A simulation's table entry held by a warp: one coalesced load of its
// words (lane l holds words l and l + 32, read through L2 so that the
// previous launch's commits are seen), fields taken by shuffles.  This
// replaces a few dozen dependent scalar loads at the start of every work
// item with one round trip.  The words a work item reads: every field up to
// `lowmach` (the counters and the commit's fields after it are not read
// through this copy).
constexpr int kSimWords = 64;
static_assert(offsetof(SimDev, lowmach) + 4 <= 4 * kSimWords && sizeof(SimDev) >= 4 * kSimWords,
              "the fields a work item reads must lie in the first 256 bytes of its table entry");
struct WarpSim {
  unsigned w0, w1;
};
__device__ __forceinline__ WarpSim load_sim(const SimDev *G, int lane) {
  const unsigned *p = reinterpret_cast<const unsigned *>(G);
  WarpSim s;
  s.w0 = __ldcg(p + lane);
  s.w1 = __ldcg(p + lane + 32);
  return s;
}
template <int I>
__device__ __forceinline__ unsigned sim_word(const WarpSim &s) {
  static_assert(I >= 0 && I < kSimWords, "word index");
  return __shfl_sync(0xffffffffu, I < 32 ? s.w0 : s.w1, I & 31);
}
template <class T, size_t OFF>
__device__ __forceinline__ T sim_get(const WarpSim &s) {
  static_assert(OFF % 4 == 0 && (sizeof(T) == 4 || sizeof(T) == 8), "field layout");
  if constexpr (sizeof(T) == 4) {
    const unsigned x = sim_word<(int)(OFF / 4)>(s);
    T v;
    memcpy(&v, &x, 4);
    return v;
  } else {
    const unsigned long long x =
        (unsigned long long)sim_word<(int)(OFF / 4)>(s) | ((unsigned long long)sim_word<(int)(OFF / 4) + 1>(s) << 32);
    T v;
    memcpy(&v, &x, 8);
    return v;
  }
}
#define FV2D_SIM(ws, field) bm::sim_get<decltype(SimDev::field), offsetof(SimDev, field)>(ws)

struct SimView {
  const float *src;
  float *dst;
  const float *rows;
  long long PL;
  int Nx, Ny, P;
  bool avg, last;
  float dt, gamma, gm1, inv_dx, inv_dy, dy, gx, gy, kappa, mu, gdx, gdy, bg_r, bg_e;
  float bctc_lo_v, bctc_hi_v;
  int bcx, bcy, grav, tc, visc, lowmach, wb, bctc_lo, bctc_hi;
};

// consToPrim of a stored offset state (States.h:32-43); the negative reset of
// checkNegatives (SimInfo.h:618-627) where the reference's Q carries it: every
// stage but the second RK2 stage, whose Q is consToPrim(U*) alone
// (Update.h:209).
__device__ __forceinline__ S4<float> to_prim(const float u[4], const SimView &S) {
  float r = u[0] + S.bg_r;
  const float uu = u[1] / r, vv = u[2] / r;
  float p = pressure_of(u[3], S.bg_e, r, uu, vv, S.gm1, S.lowmach);
  if (!S.avg) {
    if (r < 0.f) r = 1e-8f;
    if (p < 0.f) p = 1e-8f;
  }
  return S4<float>{r, uu, vv, p};
}

template <int RS>
__device__ __forceinline__ S4<float> solve(const S4<float> &qL, const S4<float> &qR, float gdx, const Gas<float> &gas,
                                           float &pout) {
  S4<float> f;
  riemann<RS>(qL, qR, f, pout, gdx, gas);
  return f;
}

// y face between a cell and the one below it (swap_component, States.h:104-110)
template <int RS>
__device__ __forceinline__ S4<float> yflux(const S4<float> &top, const S4<float> &bottom, float gdy,
                                           const Gas<float> &gas, float &pout) {
  return swap_uv(solve<RS>(swap_uv(top), swap_uv(bottom), gdy, gas, pout));
}

}  // namespace bm

// One work item (see the header comment), with the Riemann solver, the
// reconstruction and the family fixed at compile time.
template <int RS, int RECON, bool EXT>
__device__ __forceinline__ void march_item(const BatchArgs &a, const WorkItem item, const bm::WarpSim &W,
                                           const int lane) {
  using namespace bm;
  constexpr bool SLOPES = RECON != BR_PCM;
  constexpr bool MH = RECON == BR_MH;
  static_assert(EXT || (RS != RS_FSLP && !MH), "FSLP and MUSCL-Hancock are compiled in the extended family");
  SimView S;
  {
    float *U[2] = {sim_get<float *, offsetof(SimDev, U)>(W), sim_get<float *, offsetof(SimDev, U) + 8>(W)};
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
  if constexpr (EXT) {
    S.rows = FV2D_SIM(W, rows);
    S.dy = FV2D_SIM(W, dy);
    S.gdx = FV2D_SIM(W, gdx);
    S.gdy = FV2D_SIM(W, gdy);
    S.bctc_lo_v = FV2D_SIM(W, bctc_lo_v);
    S.bctc_hi_v = FV2D_SIM(W, bctc_hi_v);
    S.wb = FV2D_SIM(W, wb);
    S.bctc_lo = FV2D_SIM(W, bctc_lo);
    S.bctc_hi = FV2D_SIM(W, bctc_hi);
  } else {
    S.rows = nullptr;
    S.dy = 0.f;
    S.gdx = S.gdy = 0.f;
    S.bctc_lo_v = S.bctc_hi_v = 0.f;
    S.wb = 0;
    S.bctc_lo = S.bctc_hi = FV2D_BCTC_NONE;
  }
  const Gas<float> gas{S.gamma, S.gm1, FV2D_SIM(W, entho), FV2D_SIM(W, fslp_K)};
  const int ntiles = FV2D_SIM(W, ntx) * FV2D_SIM(W, nty);
  const int Nx = S.Nx, Ny = S.Ny;
  const int gxl = item.tx * STRIP + lane;           // padded column of this lane
  const bool colok = gxl < Nx + 4;
  const bool out_lane = lane >= 2 && lane < 30 && gxl - 2 < Nx;
  const int band = FV2D_SIM(W, band);
  const int j0 = item.ty * band, jend = min(j0 + band, Ny);  // interior rows [j0, jend)
  const float dtdx = S.dt * S.inv_dx, dtdy = S.dt * S.inv_dy;
  const float ax = 0.5f * S.dt * S.inv_dx, ay = 0.5f * S.dt * S.inv_dy;  // MUSCL-Hancock half step

  auto load = [&](int L, float u[4]) {  // padded row L
    const long long g = (long long)L * S.P + gxl;
    if (colok) {
#pragma unroll
      for (int k = 0; k < 4; ++k) u[k] = __ldg(S.src + k * S.PL + g);
    } else {
      u[0] = 1.f; u[1] = 0.f; u[2] = 0.f; u[3] = 1.f;  // never reaches an output lane
    }
  };
  const S4<float> zero4{0.f, 0.f, 0.f, 0.f};
  // y slopes from the row differences D(row) = q(row) - q(row - 1)
  auto yslope = [&](const S4<float> &dl, const S4<float> &dr) {
    if constexpr (SLOPES) return slope4(dl, dr);
    else return zero4;
  };
  auto ydiff = [&](const S4<float> &lo, const S4<float> &hi) {
    if constexpr (SLOPES) return sub4(hi, lo);
    else return zero4;
  };
  // x slope of a row: the left difference formed in every lane, the right
  // one taken from the next lane
  auto xslope = [&](const S4<float> &c) {
    if constexpr (SLOPES) {
      const S4<float> dl = sub4(c, shfl_up4(c, 1));
      return slope4(dl, shfl_down4(dl, 1));
    } else {
      return zero4;
    }
  };
  // the state the faces of a cell are reconstructed from: the cell itself,
  // or its MUSCL-Hancock predictor
  auto predict = [&](const S4<float> &q, const S4<float> &sx, const S4<float> &sy) {
    if constexpr (MH) return hancock(q, sx, sy, ax, ay, S.gamma);
    else return q;
  };

  // Rows enter the window one per iteration, through this loop only: every
  // row's primitives, slopes and MUSCL-Hancock predictor and every y face
  // come from one code path, so a face that two bands share (their boundary)
  // gets bit-identical fluxes from both and the step stays exactly
  // conservative (separately compiled copies of the same expressions may be
  // contracted into multiply-adds differently).  Iteration L loads padded row
  // L; the first four iterations only fill the window, the others update row
  // C = L - 2.  Rows are loaded one iteration ahead of their use.
  S4<float> qm = zero4, q0 = zero4, qp = zero4, Dp = zero4, h0 = zero4, hx0 = zero4, qt0 = zero4, Gm = zero4;
  float U0[4] = {0.f, 0.f, 0.f, 0.f}, Up[4] = {0.f, 0.f, 0.f, 0.f};
  float poutM = 0.f;
  float lmax = 0.f;
  unsigned nneg = 0, nnan = 0;
  float Unext[4];
  load(j0, Unext);
  for (int L = j0; L < jend + 4; ++L) {
    const int C = L - 2;
    const int j = C - 2;
    float Un[4] = {Unext[0], Unext[1], Unext[2], Unext[3]};
    if (L + 1 < jend + 4) load(L + 1, Unext);
    const S4<float> qn = to_prim(Un, S);
    const S4<float> Dn = ydiff(qp, qn);
    const S4<float> hp = yslope(Dp, Dn);  // slope of row L - 1 (from L = j0 + 2 on)
    S4<float> hxp = zero4;
    if constexpr (MH) hxp = xslope(qp);
    const S4<float> qtp = predict(qp, hxp, hp);
    float poutP = 0.f;
    S4<float> Gp = zero4;
    if (L >= j0 + 3)  // face between rows C and C + 1
      Gp = yflux<RS>(face4(qt0, h0, 0.5f), face4(qtp, hp, -0.5f), S.gdy, gas, poutP);
    if (L >= j0 + 4) {
      // x faces of row C: lane l solves face l - 1/2
      S4<float> hx;
      if constexpr (MH) hx = hx0;
      else hx = xslope(q0);
      float poutX;
      const S4<float> Fw = solve<RS>(shfl_up4(face4(qt0, hx, 0.5f), 1), face4(qt0, hx, -0.5f), S.gdx, gas, poutX);
      const S4<float> Fe = shfl_down4(Fw, 1);

      // gravity of the row: constant, or the per-row table (the analytical
      // value applies to both directions, Gravity.h:45-58)
      float g_x = S.gx, g_y = S.gy;
      if constexpr (EXT) {
        if (S.grav == BG_ROW) g_x = g_y = S.rows[j * kRowStride + ROW_G];
      }
      // well-balanced y fluxes at the y boundaries (Update.h:149-156)
      S4<float> GmU = Gm, GpU = Gp;
      if constexpr (EXT) {
        if (S.wb) {
          const float g = S.grav == BG_NONE ? 0.f : g_y;
          if (j == 0) GmU = S4<float>{0.f, 0.f, poutP - q0.r * g * S.dy, 0.f};
          if (j == Ny - 1) GpU = S4<float>{0.f, 0.f, poutM + q0.r * g * S.dy, 0.f};
        }
      }

      // update in the reference's order: x flux, x gravity, y flux, y gravity,
      // conduction, viscosity (Update.h:114-168, 176-191)
      float un[4];
      {
        const float2 d = make_float2(dtdx, dtdx);
        const S4<float> dF = sub4(Fw, Fe);
        const float2 lo = __ffma2_rn(lo2(dF), d, make_float2(U0[0], U0[1]));
        const float2 hi = __ffma2_rn(hi2(dF), d, make_float2(U0[2], U0[3]));
        un[0] = lo.x; un[1] = lo.y; un[2] = hi.x; un[3] = hi.y;
      }
      if (S.grav) {
        un[2] += S.dt * q0.r * g_x;
        un[3] += S.dt * 0.5f * (Fw.r + Fe.r) * g_x;
      }
      {
        const float2 d = make_float2(dtdy, dtdy);
        const S4<float> dG = sub4(GmU, GpU);
        const float2 lo = __ffma2_rn(lo2(dG), d, make_float2(un[0], un[1]));
        const float2 hi = __ffma2_rn(hi2(dG), d, make_float2(un[2], un[3]));
        un[0] = lo.x; un[1] = lo.y; un[2] = hi.x; un[3] = hi.y;
      }
      if (S.grav) {
        un[2] += S.dt * q0.r * g_y;
        un[3] += S.dt * 0.5f * (GmU.r + GpU.r) * g_y;
      }
      if (S.tc) {
        const float TC = q0.p / q0.r;
        const float TL = __shfl_up_sync(0xffffffffu, TC, 1), TR = __shfl_down_sync(0xffffffffu, TC, 1);
        const float TU = qm.p / qm.r, TD = qp.p / qp.r;
        float kL = S.kappa, kR = S.kappa, kU = S.kappa, kD = S.kappa;
        if constexpr (EXT) {
          if (S.tc == BK_ROW) {
            const float *rw = S.rows + j * kRowStride;
            kL = rw[ROW_KL]; kR = rw[ROW_KR]; kU = rw[ROW_KU]; kD = rw[ROW_KD];
          }
        }
        float FL = kL * (TC - TL) * S.inv_dx, FR = kR * (TR - TC) * S.inv_dx;
        const float FU = kU * (TC - TU) * S.inv_dy, FD = kD * (TD - TC) * S.inv_dy;
        if constexpr (EXT) {
          // the y-boundary modes replace the x-face fluxes FL / FR
          // (ThermalConduction.h:75-103, as the reference writes them)
          if (j == 0 && S.bctc_lo == FV2D_BCTC_FIXED_TEMPERATURE) FL = kL * 2.f * (TC - S.bctc_lo_v) * S.inv_dy;
          if (j == 0 && S.bctc_lo == FV2D_BCTC_FIXED_GRADIENT) FL = kL * S.bctc_lo_v;
          if (j == Ny - 1 && S.bctc_hi == FV2D_BCTC_FIXED_TEMPERATURE) FR = kR * 2.f * (S.bctc_hi_v - TC) * S.inv_dy;
          if (j == Ny - 1 && S.bctc_hi == FV2D_BCTC_FIXED_GRADIENT) FR = kR * S.bctc_hi_v;
        }
        un[3] += dtdx * (FR - FL) + dtdy * (FD - FU);
      }
      if (S.visc) {
        // 3x3 stencil of velocities: rows C-1, C, C+1 (qm, q0, qp) x lanes -1, 0, +1
        const float odx = S.inv_dx, ody = S.inv_dy, mu = S.mu;
        float u_[3][3], v_[3][3];
        const S4<float> *rws[3] = {&qm, &q0, &qp};
  #pragma unroll
        for (int r = 0; r < 3; ++r) {
          u_[r][1] = rws[r]->u;
          v_[r][1] = rws[r]->v;
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
        const int i = gxl - 2;
        const long long g = (long long)C * S.P + gxl;
        if (S.avg) {  // SSP-RK2: 0.5 (U^n + U**) (Update.h:214-220), offsets alike
  #pragma unroll
          for (int k = 0; k < 4; ++k) un[k] = 0.5f * (S.dst[k * S.PL + g] + un[k]);
        }
  #pragma unroll
        for (int k = 0; k < 4; ++k) S.dst[k * S.PL + g] = un[k];
        if (S.last) {
          // primitive state of the new cell for the next dt, negative guard
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
              const long long gg = (long long)(ty[b] + 2) * S.P + (tx[c] + 2);
              S.dst[gg] = un[0];
              S.dst[S.PL + gg] = nx[c] ? -un[1] : un[1];
              S.dst[2 * S.PL + gg] = ny[b] ? -un[2] : un[2];
              S.dst[3 * S.PL + gg] = un[3];
            }
        }
      }

    }  // L >= j0 + 4

    // advance the window
    qm = q0;
    q0 = qp;
    qp = qn;
    h0 = hp;
    Dp = Dn;
    if constexpr (MH) hx0 = hxp;
    qt0 = qtp;
    Gm = Gp;
    poutM = poutP;
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
    if (S.last) atomicMax(&Gw->acc_bits, __float_as_uint(lmax));
    if (wn) atomicAdd(&Gw->negatives, (unsigned long long)wn);
    if (wnan) atomicAdd(&Gw->nan_cells, wnan);
    __threadfence();
    const unsigned t = atomicAdd(&Gw->ticket, 1u);
    if (t == (unsigned)ntiles - 1u) commit_stage(Gw);
  }
}

// The plain and diffusive families: HLL / HLLC x PCM / PLM.
template <int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB) batch_march_kernel(const BatchArgs a) {
  const int lane = threadIdx.x & 31;
  const int nwarps = gridDim.x * (NT / 32);
  const int nw = *a.n_work;
  for (int w = blockIdx.x * (NT / 32) + (threadIdx.x >> 5); w < nw; w += nwarps) {
    const WorkItem item = a.work[w];
    // the table changes between launches (commits, admissions), not during
    // a simulation's items of one launch
    const bm::WarpSim W = bm::load_sim(a.sims + item.sim, lane);
    if (FV2D_SIM(W, status) != SIM_ACTIVE) continue;
    const bool plm = FV2D_SIM(W, recon) == BR_PLM;
    if (FV2D_SIM(W, rs) == RS_HLL) {
      if (plm)
        march_item<RS_HLL, BR_PLM, false>(a, item, W, lane);
      else
        march_item<RS_HLL, BR_PCM, false>(a, item, W, lane);
    } else {
      if (plm)
        march_item<RS_HLLC, BR_PLM, false>(a, item, W, lane);
      else
        march_item<RS_HLLC, BR_PCM, false>(a, item, W, lane);
    }
    __syncwarp();
  }
}

template <int RS>
__device__ __forceinline__ void march_ext_recon(const BatchArgs &a, const WorkItem item, const bm::WarpSim &W,
                                                const int lane) {
  const int recon = FV2D_SIM(W, recon);
  if (recon == BR_MH)
    march_item<RS, BR_MH, true>(a, item, W, lane);
  else if (recon == BR_PLM)
    march_item<RS, BR_PLM, true>(a, item, W, lane);
  else
    march_item<RS, BR_PCM, true>(a, item, W, lane);
}

// The extended family: HLL / HLLC / FSLP x PCM / PLM / MUSCL-Hancock, with
// the per-row tables and the boundary fluxes.
template <int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB) batch_march_ext_kernel(const BatchArgs a) {
  const int lane = threadIdx.x & 31;
  const int nwarps = gridDim.x * (NT / 32);
  const int nw = *a.n_work;
  for (int w = blockIdx.x * (NT / 32) + (threadIdx.x >> 5); w < nw; w += nwarps) {
    const WorkItem item = a.work[w];
    const bm::WarpSim W = bm::load_sim(a.sims + item.sim, lane);
    if (FV2D_SIM(W, status) != SIM_ACTIVE) continue;
    const int rs = FV2D_SIM(W, rs);
    if (rs == RS_HLL)
      march_ext_recon<RS_HLL>(a, item, W, lane);
    else if (rs == RS_FSLP)
      march_ext_recon<RS_FSLP>(a, item, W, lane);
    else
      march_ext_recon<RS_HLLC>(a, item, W, lane);
    __syncwarp();
  }
}

}  // namespace fv2d
