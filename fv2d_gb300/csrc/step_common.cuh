// step_common.cuh -- data structures shared by the host API and the FP64
// kernels of the plain (drop-in) path.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace fv2d {

// Tile of interior cells owned by one CTA of the fused step kernel.
constexpr int TX = 16;  // cells along x (even: TMA rows start on 16-byte boundaries)
constexpr int TY = 16;  // cells along y
constexpr int HALO = 2; // ghost depth read by PLM + the 3x3 viscous stencil
constexpr int SW = TX + 2 * HALO;  // staged tile width  (TMA box x)
constexpr int SH = TY + 2 * HALO;  // staged tile height (TMA box y)
constexpr int NT = 288;            // threads per CTA (9 warps: the 544 faces of a tile in two rounds)

enum { RECON_PCM = 0, RECON_PLM = 2, RECON_MH = 3 };
enum { STAGE_EULER = 0, STAGE_RK2_PREDICT = 1, STAGE_RK2_CORRECT = 2 };
enum { RUN_RUNNING = 0, RUN_DONE = 1, RUN_SAVE = 2, RUN_NUMERIC = 3, RUN_PAUSED = 4 };
enum { DEVERR_TMA_TIMEOUT = 1, DEVERR_BOUNDS = 2 };

// Simulation clock, dt and reduction accumulators, resident in device memory.
// Written by the last CTA of each step (or by the set-up pass), read by the
// next launch: kernels never exchange these within a launch.
struct DevState {
  double t;          // time after the last committed update (main.cpp:83)
  double dt;         // CFL dt of the current primitive state (ComputeDt.h:64)
  double inv_hyp;    // max inverse hyperbolic dt of the current state
  double last_dt;    // dt used by the last update
  double tend, next_save, eps;  // device-driven loop control
  unsigned long long acc_hyp;   // running max (bits of a non-negative double)
  unsigned long long cnt_acc[3];
  unsigned long long counters[3];  // checkNegatives counts of the last update
  int parity;        // which primitive buffer holds the current state
  int ite;           // committed updates
  int status;        // RUN_*
  int check_save;    // stop before an iteration that must write a snapshot
  int steps_in_call; // iterations done by the current fv2d_advance
  int max_steps;     // iteration cap of the current fv2d_advance
  int log_cap;       // capacity of the per-iteration log (records)
  int error;         // DEVERR_* bit set by a kernel that gave up waiting
  unsigned int ticket;  // CTAs finished in the running launch
  int pad;
};

// Everything one step launch needs besides the two tensor maps.
struct StepArgs {
  double *Q[2];       // primitive planes (4 planes, ghosts included)
  double *U;          // conservative planes (same layout)
  double *U1;         // RK2 predictor planes (same layout)
  const float *grav_row;  // analytical gravity per interior row (float, Gravity.h:16)
  const double *kap_row;  // per interior row: kappaL, kappaR, kappaU, kappaD
  DevState *st;
  double *log;        // per-iteration records {t, dt, inv_hyp, 3 counters} (may be null)
  long long plane;    // elements per field plane
  int pitch;          // elements per padded row
  int Nx, Ny;
  int nblocks;
  int stage;          // STAGE_*
  int driven;         // 1: dt and loop control from DevState
  double dt_arg;      // dt when driven == 0
  // gas and mesh constants
  double gamma, gm1, entho, fslp_K;
  double dx, dy, inv_dx, inv_dy;
  int dx_pow2, dy_pow2;  // 1/dx (1/dy) is exact: divisions become products
  uint64_t rw_dx, rw_dy;  // otherwise quotients by dx (dy) share its reciprocal word
  double one_over_dx, one_over_dy;  // 1.0/dx, 1.0/dy (Viscosity.h:57-58)
  double gx_dx, gy_dy;  // FSLP gravity terms gx*dx, gy*dy (Update.h:119)
  double gxf, gyf;      // constant gravity narrowed to float (Gravity.h:39)
  double eps_reset;     // epsilon_reset_negative
  double CFL, inv_tc, inv_visc;  // dt finalisation (ComputeDt.h:64)
  double mu;
  double bctc_ymin_value, bctc_ymax_value;
  int bcx, bcy;
  int grav_mode;  // 0 none, 1 constant, 2 analytical
  int tc, visc, wb;
  int bctc_ymin, bctc_ymax;
  double *mirror;  // device view of a page-locked host (Ny x Nx x 4) array that the
                   // final stage also writes the new primitives to (may be null)
};

// Set-up pass arguments (interior upload -> planes, ghosts, U, dt reduction).
struct PrepArgs {
  const double *q_aos;  // interior primitives, interleaved (Ny x Nx x 4)
  double *Q;            // destination primitive planes (current buffer)
  double *U;
  DevState *st;
  long long plane;
  int pitch, Nx, Ny, nblocks;
  double gamma, gm1, dx, dy, inv_dx, inv_dy;
  int dx_pow2, dy_pow2;
  uint64_t rw_dx, rw_dy;
  double CFL, inv_tc, inv_visc;
  int bcx, bcy;
};

}  // namespace fv2d
