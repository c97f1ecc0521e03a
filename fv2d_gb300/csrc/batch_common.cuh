// batch_common.cuh -- data structures of the batched FP32 service (many
// independent simulations of different sizes advanced together).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace fv2d {

enum { SIM_FREE = 0, SIM_ACTIVE = 1, SIM_DONE = 2, SIM_FAILED = 3 };

// One simulation resident in HBM.  Conservative state in binary32, two
// buffers (the step reads one and writes the other, ghost ring included so
// that every tile stages its halo with one TMA load), clock and dt in
// binary64.  64-byte aligned: the device reads it field by field.
struct __align__(64) SimDev {
  float *U[2];          // 4 planes each: rho, rho u, rho v, E; (N + 4) rows x pitch
  long long plane;      // floats per plane
  int pitch;            // floats per padded row
  int N;                // N x N interior cells
  int ntx, nty;         // tiles along x and y (for the kernel's bucket)
  int cur;              // buffer holding the current state
  int status;           // SIM_*
  int step, max_steps;  // committed steps, stop after max_steps
  double t, dt, tend;   // binary64 clock (stop when t + eps >= tend)
  double eps;
  double inv_tc, inv_visc, cfl;  // dt finalisation (ComputeDt.h:64)
  float gamma, gm1, entho;
  float dx, dy, inv_dx, inv_dy;
  float gx, gy, kappa, mu;
  int rs;               // Riemann solver (RS_HLL / RS_HLLC)
  int recon;            // 0 PCM, 2 PLM
  int bcx, bcy;
  int grav, tc, visc;
  int lowmach;          // recover p = (E - Ek)(gamma - 1) in binary64 where it cancels
  unsigned int acc_bits;  // running max of the inverse hyperbolic dt (float bits)
  unsigned int ticket;    // tiles finished in the running launch
  unsigned long long negatives;  // cells reset by the negative guard (all steps)
  int tma_ok;           // tensor map valid for this simulation
  unsigned int nan_cells;  // NaN cells produced by the running step: the commit fails the simulation
};

// Pressure (E - rho |u|^2 / 2)(gamma - 1) of the binary32 state.  Low-Mach
// requests recover it in binary64 where it cancels: when the kinetic energy is
// more than a quarter of E the subtraction loses two or more bits.  Elsewhere
// the binary32 evaluation is within a unit or two of the binary64 one rounded
// to binary32, so the binary64 pipe (1/64 of the FP32 rate) is not used.
__device__ __forceinline__ float pressure_of(float E, float r, float u, float v, float gm1, int lowmach) {
  const float ek = 0.5f * r * (u * u + v * v);
  if (lowmach && fabsf(ek) > 0.25f * fabsf(E)) {
    const double rd = r, ud = u, vd = v;
    return (float)(((double)E - 0.5 * rd * (ud * ud + vd * vd)) * (double)gm1);
  }
  return (E - ek) * gm1;
}

__device__ __forceinline__ bool is_nan_f(float x) { return (__float_as_uint(x) & 0x7FFFFFFFu) > 0x7F800000u; }

// A tile of one simulation: sim index in the table, tile coordinates.
struct WorkItem {
  int sim;
  short tx, ty;
};

struct BatchArgs {
  SimDev *sims;
  const WorkItem *work;
  const int *n_work;            // device-resident count (work list changes between replays)
  const CUtensorMap *tmaps;     // per simulation, per buffer: tmaps[2 * sim + buf] (global memory)
};

}  // namespace fv2d
