// ic.h -- initial conditions of the fv2d problems, one source for host code
// (binary64 with libm, the plain path: problems.cpp) and device code (the
// batched service builds its initial states on the GPU).
#pragma once

#include <math.h>
#include <stdint.h>

#include "../../include/fv2d_types.h"

#ifdef __CUDACC__
#define FV2D_HD __host__ __device__
#else
#define FV2D_HD
#endif

namespace fv2d {

// SplitMix64 finaliser (Steele, Lea, Flood 2014).
FV2D_HD inline uint64_t splitmix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

// Counter-based uniform draw in [0, 1) of (seed, cell, stream).
FV2D_HD inline double uniform01(int32_t seed, int64_t cell, int32_t stream) {
  uint64_t key = ((uint64_t)(uint32_t)seed << 32) ^ ((uint64_t)cell * 4u + (uint64_t)(uint32_t)stream);
  return (double)(splitmix64(key) >> 11) * 0x1.0p-53;
}

// Initial conditions of Init.h:17-265 (interior cells; unset fields stay at
// the zero the reference's Views start with), plus the extension problems.
FV2D_HD inline void init_cell(const fv2d_params &p, int problem, int i, int j, double *q) {
  const double dx = (p.xmax - p.xmin) / p.Nx, dy = (p.ymax - p.ymin) / p.Ny;
  // SimInfo.h:494-499 with ibeg = jbeg = Nghosts; i, j are interior indices
  const double x = p.xmin + ((double)i + 0.5) * dx, y = p.ymin + ((double)j + 0.5) * dy;
  const double xmid = 0.5 * (p.xmin + p.xmax), ymid = 0.5 * (p.ymin + p.ymax);
  const int64_t cell = (int64_t)j * p.Nx + i;
  q[0] = q[1] = q[2] = q[3] = 0.0;
  switch (problem) {
    case FV2D_PB_SOD_X:  // Init.h:20-35
    case FV2D_PB_SOD_Y:  // Init.h:83-98
    {
      const double c = (problem == FV2D_PB_SOD_X) ? x : y;
      const bool left = c <= 0.5;
      q[0] = left ? p.sod_rho_left : p.sod_rho_right;
      q[3] = left ? p.sod_p_left : p.sod_p_right;
      q[1] = 0.0;
      break;
    }
    case FV2D_PB_GRESHO_VORTEX: {  // Init.h:42-78
      const double xr = x - xmid, yr = y - ymid;
      const double r = sqrt(xr * xr + yr * yr);
      const double p0 = p.gresho_density / (p.gamma0 * p.gresho_Mach * p.gresho_Mach);
      q[0] = p.gresho_density;
      double u_phi;
      if (r < 0.2) {
        u_phi = 5.0 * r;
        q[3] = p0 + 12.5 * r * r;
      } else if (r < 0.4) {
        u_phi = 2.0 - 5.0 * r;
        q[3] = p0 + 12.5 * r * r + 4.0 * (1.0 - 5.0 * r + log(5.0 * r));
      } else {
        u_phi = 0.0;
        q[3] = p0 - 2.0 + 4.0 * log(2.0);
      }
      const double xnr = xr / r, ynr = yr / r;
      q[1] = -ynr * u_phi;
      q[2] = xnr * u_phi;
      break;
    }
    case FV2D_PB_BLAST: {  // Init.h:103-131
      const double xr = xmid - x, yr = ymid - y;
      const double r = sqrt(xr * xr + yr * yr);
      const bool in = r < 0.2;
      q[0] = in ? 1.0 : 1.2;
      q[3] = in ? 10.0 : 0.1;
      break;
    }
    case FV2D_PB_H84: {  // Init.h:136-154; the random pool is a counter-based generator here
      q[0] = pow(y, p.m1);
      q[3] = pow(y, p.m1 + 1.0);
      q[2] = p.h84_pert * (-0.5 + uniform01(p.seed, cell, 0));
      break;
    }
    case FV2D_PB_C91: {  // Init.h:159-180
      const double T = (1.0 + p.theta1 * y);
      const double pert = p.c91_pert * (-0.5 + uniform01(p.seed, cell, 0));
      q[0] = pow(T, p.m1);
      q[3] = pow(T, p.m1 + 1.0) * (1.0 + pert);
      break;
    }
    case FV2D_PB_DIFFUSION: {  // Init.h:185-206
      const double x0 = (x - xmid), y0 = (y - ymid);
      const double r = sqrt(x0 * x0 + y0 * y0);
      q[0] = (r < 0.2) ? 1.0 : 0.1;
      q[1] = 1.0; q[2] = 1.0; q[3] = 1.0;
      break;
    }
    case FV2D_PB_RAYLEIGH_TAYLOR: {  // Init.h:211-237
      const double P0 = 2.5;
      q[0] = (y < ymid) ? 1.0 : 2.0;
      q[3] = P0 + 0.1 * p.gy * y;
      if (y > -1.0 / 3.0 && y < 1.0 / 3.0)
        q[2] = 0.01 * (1.0 + cos(4 * M_PI * x)) * (1 + cos(3.0 * M_PI * y)) / 4.0;
      break;
    }
    case FV2D_PB_KELVIN_HELMHOLTZ: {  // Init.h:245-265
      const double q1 = tanh((y - p.kh_y1) / p.kh_a);
      const double q2 = tanh((y - p.kh_y2) / p.kh_a);
      const double s2 = p.kh_sigma * p.kh_sigma;
      const double dy1 = (y - p.kh_y1) * (y - p.kh_y1);
      const double dy2 = (y - p.kh_y2) * (y - p.kh_y2);
      q[0] = 1.0 + p.kh_rho_fac * 0.5 * (q1 - q2);
      q[1] = p.kh_uflow * (q1 - q2 - 1.0);
      q[2] = p.kh_amp * sin(2.0 * M_PI * x) * (exp(-dy1 / s2) + exp(-dy2 / s2));
      q[3] = p.kh_P0;
      break;
    }
    case FV2D_PB_SEDOV: {
      const double xr = x - xmid, yr = y - ymid;
      const double r = sqrt(xr * xr + yr * yr);
      q[0] = p.sedov_rho;
      q[3] = (r <= p.sedov_r0) ? (p.gamma0 - 1.0) * p.sedov_E0 / (M_PI * p.sedov_r0 * p.sedov_r0) : p.sedov_p_ambient;
      break;
    }
    case FV2D_PB_KH_STEP: {
      const bool in = fabs(y - ymid) < 0.25;
      q[0] = in ? p.khs_rho_in : p.khs_rho_out;
      q[1] = (in ? p.khs_u : -p.khs_u) + p.khs_noise * (2.0 * uniform01(p.seed, cell, 1) - 1.0);
      q[2] = p.khs_amp * sin(4.0 * M_PI * x) + p.khs_noise * (2.0 * uniform01(p.seed, cell, 2) - 1.0);
      q[3] = p.khs_p0;
      break;
    }
    case FV2D_PB_RT_HYDROSTATIC: {
      const double rho = (y > p.rt_y_interface) ? p.rt_rho_top : p.rt_rho_bottom;
      q[0] = rho;
      q[2] = p.rt_amp * (1.0 + cos(4.0 * M_PI * x)) * (1.0 + cos(3.0 * M_PI * (y - p.rt_y_interface))) / 4.0;
      q[3] = p.rt_p_interface + rho * p.gy * (y - p.rt_y_interface);
      break;
    }
    default:
      break;
  }
}

}  // namespace fv2d
