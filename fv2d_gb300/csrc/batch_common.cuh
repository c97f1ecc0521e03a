// batch_common.cuh -- data structures of the batched FP32 service (many
// independent simulations of different sizes advanced together).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/fv2d_types.h"

namespace fv2d {

enum { SIM_FREE = 0, SIM_ACTIVE = 1, SIM_DONE = 2, SIM_FAILED = 3 };

// Reconstructions of the served step (the values of fv2d_params.reconstruction
// they come from: PCM and PCM_WB -> PCM, PLM, MUSCL_HANCOCK).
enum { BR_PCM = 0, BR_PLM = 2, BR_MH = 3 };
// Kernel families of the served step (bit f of a configuration's family
// mask: it runs requests of family f): plain hydro (HLL / HLLC, PCM / PLM,
// constant gravity), diffusive (the same with constant conduction and / or
// viscosity), extended (FSLP, MUSCL-Hancock, per-row tables, boundary
// fluxes).
enum { FAM_PLAIN = 0, FAM_DIFF = 1, FAM_EXT = 2, kFamilies = 3 };
// Gravity and conductivity forms of the served step.
enum { BG_NONE = 0, BG_CONST = 1, BG_ROW = 2 };  // BG_ROW: per-row table (analytical gravity)
enum { BK_NONE = 0, BK_CONST = 1, BK_ROW = 2 };  // BK_ROW: per-row face conductivities (B02)

// Per-row table of a simulation (floats, kRowStride per interior row):
// gravity of the row (Gravity.h:15-57 narrowed to float) and the face
// conductivities kappaL, kappaR, kappaU, kappaD (ThermalConduction.h:46-53).
enum { ROW_G = 0, ROW_KL = 1, ROW_KR = 2, ROW_KU = 3, ROW_KD = 4 };
constexpr int kRowStride = 8;

// One simulation resident in HBM.  Conservative state in binary32 stored as
// the offset from a per-simulation background (rho - bg_r, rho u, rho v,
// E - bg_e): where the state stays near its background the stored words keep
// more of its digits.  Two buffers (a stage reads one and writes the other,
// ghost ring included so that every tile stages its halo with one TMA load),
// clock and dt in binary64.  64-byte aligned: the device reads it field by
// field.
struct __align__(64) SimDev {
  float *U[2];          // 4 planes each: rho, rho u, rho v, E offsets; (Ny + 4) rows x pitch
  const float *rows;    // per-row table (Ny x kRowStride), or null
  long long plane;      // floats per plane
  int pitch;            // floats per padded row
  int Nx, Ny;           // interior cells
  int ntx, nty;         // work items along x and y (for the kernel configuration of its lane)
  int band;             // rows per work item: the tile height, or the march kernels' band (chosen per lane)
  int cur;              // buffer holding the current state
  int status;           // SIM_*
  int step, max_steps;  // committed steps, stop after max_steps
  int ts, stage;        // time stepping (0 Euler, 1 SSP-RK2) and the stage the next launch runs
  double t, dt, tend;   // binary64 clock (stop when t + eps >= tend)
  double eps;
  double inv_tc, inv_visc, cfl;  // dt finalisation (ComputeDt.h:64)
  float gamma, gm1, entho, fslp_K;
  float dx, dy, inv_dx, inv_dy;
  float gx, gy, kappa, mu;
  float gdx, gdy;       // FSLP gravity terms gx * dx, gy * dy (Update.h:118)
  float bg_r, bg_e;     // background density and total energy of the stored offsets
  float bctc_lo_v, bctc_hi_v;  // y-boundary conduction values (ThermalConduction.h:75-103)
  int rs;               // Riemann solver (RS_HLL / RS_HLLC / RS_FSLP)
  int recon;            // BR_*
  int ext;              // 1: extended kernel family (FSLP, MUSCL-Hancock, per-row tables, boundary fluxes)
  int bcx, bcy;
  int grav, tc, visc;   // BG_*, BK_*, 0/1
  int wb;               // well-balanced y flux at the y boundaries (Update.h:149-156)
  int bctc_lo, bctc_hi; // FV2D_BCTC_* at ymin, ymax
  int lowmach;          // recover p = (E - Ek)(gamma - 1) in binary64 where it cancels
  unsigned int acc_bits;  // running max of the inverse hyperbolic dt (float bits)
  unsigned int ticket;    // work items finished in the running launch
  unsigned long long negatives;  // cells reset by the negative guard (all steps)
  int tma_ok;           // tensor map valid for this simulation
  unsigned int nan_cells;  // NaN cells produced by the running step: the commit fails the simulation
  unsigned int dev_err;    // BATCH_ERR_* bits of a kernel that gave up waiting: the commit fails the simulation
};

// Pressure (E - rho |u|^2 / 2)(gamma - 1) of a cell whose total energy is
// stored as the offset dE = E - bg_e: the kinetic energy is subtracted from
// the offset first, so where both are small against the background they
// cancel in full precision.  Low-Mach requests recover it in binary64 where
// it cancels (the kinetic energy more than a quarter of E: the subtraction
// loses two or more bits).  Elsewhere the binary32 evaluation is within a
// unit or two of the binary64 one rounded to binary32, so the binary64 pipe
// (1/64 of the FP32 rate) is not used.
// Every operation is an explicitly rounded intrinsic, which the compiler
// never contracts into a multiply-add: each inlined copy of this function
// gives the same bits for the same operands (kernels that evaluate a row in
// two code paths rely on that).
__device__ __forceinline__ float pressure_of(float dE, float bg_e, float r, float u, float v, float gm1,
                                             int lowmach) {
  const float ek = __fmul_rn(__fmul_rn(0.5f, r), __fadd_rn(__fmul_rn(u, u), __fmul_rn(v, v)));
  if (lowmach && fabsf(ek) > __fmul_rn(0.25f, fabsf(__fadd_rn(dE, bg_e)))) {
    const double rd = r, ud = u, vd = v;
    const double ekd = __dmul_rn(__dmul_rn(0.5, rd), __dadd_rn(__dmul_rn(ud, ud), __dmul_rn(vd, vd)));
    return (float)__dmul_rn(__dadd_rn(__dsub_rn((double)dE, ekd), (double)bg_e), (double)gm1);
  }
  return __fmul_rn(__fadd_rn(__fsub_rn(dE, ek), bg_e), gm1);
}

__device__ __forceinline__ bool is_nan_f(float x) { return (__float_as_uint(x) & 0x7FFFFFFFu) > 0x7F800000u; }

// A work item of one simulation: sim index in the table, item coordinates.
struct WorkItem {
  int sim;
  short tx, ty;
};

struct BatchArgs {
  SimDev *sims;
  const WorkItem *work;
  const int *n_work;            // device-resident count (work list changes between replays)
  const CUtensorMap *tmaps;     // per simulation, per buffer: tmaps[2 * sim + buf] (global memory)
  // ctl[0]: fault bits, set when a CTA had to stop with a tile copy still in
  // flight (the host stops the service); ctl[1]: polls of a tile copy's
  // barrier before the simulation it belongs to is failed
  unsigned int *ctl;
};

// Polls of the second, final wait for a tile copy that outlived ctl[1].
constexpr unsigned int kTileWaitFinal = 1u << 24;
// BATCH_ERR_FAMILY: a request reached a kernel built without its family's
// terms (the service's lanes keep that from happening).
enum { BATCH_ERR_TMA_TIMEOUT = 1, BATCH_ERR_FAMILY = 2 };

// Source and destination buffers of the stage a launch runs: Euler and the
// first SSP-RK2 stage read the current buffer and write the other one; the
// second RK2 stage reads the first stage's result and writes the average
// 0.5 (U^n + U**) back into the current buffer (Update.h:197-220), reading
// U^n there only at the cell it writes.
struct StageBuffers {
  const float *src;
  float *dst;
  bool avg;     // second RK2 stage: average with dst's own cell
  bool last;    // the step's last stage: dt reduction, negative guard counts and commit
};
__device__ __forceinline__ StageBuffers stage_buffers(float *const U[2], int cur, int ts, int stage) {
  StageBuffers b;
  const bool second = ts == 1 && stage == 1;
  b.src = second ? U[1 - cur] : U[cur];
  b.dst = second ? U[cur] : U[1 - cur];
  b.avg = second;
  b.last = ts == 0 || second;
  return b;
}

// The commit of one stage of a simulation, run by the thread that finished
// the simulation's last work item of the launch (ComputeDt.h:64, main.cpp:62,
// 83).  The first RK2 stage only hands over to the second; the last stage
// advances the binary64 clock, takes the next dt from the reduced inverse
// hyperbolic dt and the parabolic limits, flips the buffers after an Euler
// step and applies the stop and failure tests.
__device__ __forceinline__ void commit_stage(SimDev *Gw) {
  __threadfence();
  volatile SimDev *V = Gw;
  if (V->ts == 1 && V->stage == 0) {
    V->stage = 1;
    V->acc_bits = 0u;
    if (V->nan_cells || V->dev_err) V->status = SIM_FAILED;
    V->nan_cells = 0u;
    __threadfence();
    V->ticket = 0u;
    return;
  }
  const double ih = (double)__uint_as_float(atomicAdd(&Gw->acc_bits, 0u));
  double m = ih;
  if (m < V->inv_tc) m = V->inv_tc;
  if (m < V->inv_visc) m = V->inv_visc;
  const double dtn = V->cfl / m;
  const double t_new = V->t + V->dt;
  const int step = V->step + 1;
  V->t = t_new;
  V->step = step;
  if (V->ts == 0) V->cur = 1 - V->cur;
  V->stage = 0;
  V->dt = dtn;
  V->acc_bits = 0u;
  int status = SIM_ACTIVE;
  if (!(dtn > 0.0) || isinf(dtn) || V->nan_cells || V->dev_err)  // NaN / dt / wait guards fail this request only
    status = SIM_FAILED;
  else if (step >= V->max_steps || !(t_new + V->eps < V->tend))
    status = SIM_DONE;
  V->status = status;
  V->nan_cells = 0u;
  __threadfence();
  V->ticket = 0u;
}

}  // namespace fv2d
