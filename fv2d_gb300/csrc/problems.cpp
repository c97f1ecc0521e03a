// problems.cpp -- host-side (binary64, libm) parts of the plain path that
// depend only on parameters and positions: the reference's effective default
// parameters, the initial conditions, and the per-row gravity and
// conductivity tables.  Computing these on the host keeps transcendental
// functions (sin, cos, tanh, exp, log, pow) out of the device step and gives
// exactly the values a CPU build of the reference computes.
#include "problems.h"

#include <cmath>
#include <cstring>
#include <limits>

namespace fv2d {

namespace {
inline double f32(double x) { return (double)(float)x; }

// SimInfo.h:494-499 with ibeg = jbeg = Nghosts; i, j are interior indices.
inline double pos_x(const fv2d_params &p, double dx, int i) { return p.xmin + ((double)i + 0.5) * dx; }
inline double pos_y(const fv2d_params &p, double dy, int j) { return p.ymin + ((double)j + 0.5) * dy; }

}  // namespace

void params_default(fv2d_params *p) {
  std::memset(p, 0, sizeof(*p));
  p->struct_size = sizeof(fv2d_params);
  // [mesh] SimInfo.h:360-366
  p->Nx = 32; p->Ny = 32; p->Nghosts = 2;
  p->xmin = 0.0; p->xmax = 1.0; p->ymin = 0.0; p->ymax = 1.0;
  // [solvers] / [run] SimInfo.h:378-389, 536-545
  p->CFL = f32(0.8);
  p->boundary_x = FV2D_BC_REFLECTING; p->boundary_y = FV2D_BC_REFLECTING;
  p->reconstruction = FV2D_PCM;
  p->riemann_solver = FV2D_HLLC;
  p->time_stepping = FV2D_TS_EULER;
  p->tend = 1.0; p->save_freq = f32(1.0e-1);
  // [physics] / [misc] SimInfo.h:392-399, 549-551
  p->epsilon = f32(1.0e-6);
  p->gamma0 = f32(5.0 / 3.0);
  p->m1 = 1.0; p->theta1 = 10.0; p->m2 = 1.0; p->theta2 = 10.0;
  p->well_balanced_flux_at_y_bc = 0;
  p->fslp_K = f32(1.1);
  p->seed = 12345; p->log_frequency = 10; p->epsilon_reset_negative = f32(1.0e-8);
  // [gravity] SimInfo.h:405-411
  p->gravity_mode = FV2D_GRAV_NONE; p->gx = 0.0; p->gy = 0.0;
  p->analytical_gravity_mode = FV2D_AGM_HOT_BUBBLE; p->hot_bubble_g0 = 0.0;
  // [thermal_conduction] SimInfo.h:414-427
  p->thermal_conductivity_active = 0; p->thermal_conductivity_mode = FV2D_TCM_CONSTANT; p->kappa = 0.0;
  p->bctc_ymin = FV2D_BCTC_NONE; p->bctc_ymax = FV2D_BCTC_NONE;
  p->bctc_ymin_value = 1.0; p->bctc_ymax_value = 1.0;
  // [viscosity] SimInfo.h:430-435
  p->viscosity_active = 0; p->viscosity_mode = FV2D_VSC_CONSTANT; p->mu = 0.0;
  // problems SimInfo.h:438-458
  p->h84_pert = f32(1.0e-4); p->c91_pert = f32(1.0e-3);
  p->kh_a = f32(0.05); p->kh_amp = f32(0.01); p->kh_P0 = 1.0; p->kh_rho_fac = 0.0; p->kh_sigma = f32(0.2);
  p->kh_uflow = 1.0; p->kh_y1 = 0.5; p->kh_y2 = 1.5;
  p->gresho_density = 1.0; p->gresho_Mach = f32(0.1);
  // extension problems
  p->sod_rho_left = 1.0; p->sod_p_left = 1.0; p->sod_rho_right = 0.125; p->sod_p_right = 0.1;
  p->sedov_E0 = 1.0; p->sedov_r0 = 0.02; p->sedov_p_ambient = 1.0e-5; p->sedov_rho = 1.0;
  p->khs_rho_in = 2.0; p->khs_rho_out = 1.0; p->khs_u = 0.5; p->khs_p0 = 2.5; p->khs_amp = 0.01; p->khs_noise = 1.0e-3;
  p->rt_rho_top = 2.0; p->rt_rho_bottom = 1.0; p->rt_p_interface = 2.5; p->rt_y_interface = 0.75; p->rt_amp = 0.01;
}

bool problem_valid(int pb) {
  return (pb >= FV2D_PB_SOD_X && pb <= FV2D_PB_GRESHO_VORTEX) || pb == FV2D_PB_SEDOV || pb == FV2D_PB_KH_STEP ||
         pb == FV2D_PB_RT_HYDROSTATIC;
}

// Gravity.h:15-28: hot-bubble gravity of interior row j, narrowed to float.
float analytical_gravity_row(const fv2d_params &p, int j) {
  const double dy = (p.ymax - p.ymin) / p.Ny;
  const double y = pos_y(p, dy, j);
  const double g = p.hot_bubble_g0 * std::sin(y * M_PI * 2.0 / p.ymax);
  return (float)g;
}

// ThermalConduction.h:8-26 for a padded row index jj (ibeg = jbeg = Nghosts).
static double kappa_at(const fv2d_params &p, int jj) {
  if (p.thermal_conductivity_mode == FV2D_TCM_B02) {
    const double dy = (p.ymax - p.ymin) / p.Ny;
    const double y = p.ymin + (jj - p.Nghosts + 0.5) * dy;
    const double tr = (std::tanh((y - p.b02_ymid) / p.b02_thickness) + 1.0) * 0.5;
    return p.kappa * (p.b02_kappa1 * (1.0 - tr) + p.b02_kappa2 * tr);
  }
  return p.kappa;
}

// ThermalConduction.h:46-53: face conductivities of interior row j.  The
// reference evaluates the neighbour conductivity at the physical coordinates
// converted to int; only the row argument matters for every mode.
void kappa_row(const fv2d_params &p, int j, double out[4]) {
  const double dx = (p.xmax - p.xmin) / p.Nx, dy = (p.ymax - p.ymin) / p.Ny;
  const int jj = j + p.Nghosts;
  const double x = pos_x(p, dx, 0), y = pos_y(p, dy, j);
  (void)x;
  const double kC = kappa_at(p, jj);
  out[0] = 0.5 * (kC + kappa_at(p, (int)y));
  out[1] = 0.5 * (kC + kappa_at(p, (int)y));
  out[2] = 0.5 * (kC + kappa_at(p, (int)(y - dy)));
  out[3] = 0.5 * (kC + kappa_at(p, (int)(y + dy)));
}

// ComputeDt.h:36-44: state-independent parabolic inverse time steps.
void parabolic_inv_dt(const fv2d_params &p, double *inv_tc, double *inv_visc) {
  const double dx = (p.xmax - p.xmin) / p.Nx, dy = (p.ymax - p.ymin) / p.Ny;
  double tc = p.epsilon, visc = p.epsilon;
  if (p.thermal_conductivity_active) {
    tc = std::numeric_limits<double>::lowest();  // Kokkos::Max identity
    for (int j = 0; j < p.Ny; ++j) {
      const double k = kappa_at(p, j + p.Nghosts);
      tc = std::fmax(tc, std::fmax(2.0 * k / (dx * dx), 2.0 * k / (dy * dy)));
    }
  }
  if (p.viscosity_active) visc = std::fmax(2.0 * p.mu / (dx * dx), 2.0 * p.mu / (dy * dy));
  *inv_tc = tc;
  *inv_visc = visc;
}

const char *validate(const fv2d_params &p) {
  if (p.struct_size != sizeof(fv2d_params)) return "fv2d_params.struct_size does not match this library";
  if (p.Nx < 2 || p.Ny < 2) return "Nx and Ny must be at least 2";
  if (p.Nghosts < 2) return "Nghosts must be at least 2 (PLM and the viscous stencil read two ghost layers)";
  if ((long long)p.Nx * p.Ny > (1LL << 31)) return "grid too large";
  if (!(p.xmax > p.xmin) || !(p.ymax > p.ymin)) return "empty domain";
  if (p.boundary_x < 0 || p.boundary_x > 2 || p.boundary_y < 0 || p.boundary_y > 2) return "bad boundary type";
  if (p.reconstruction < 0 || p.reconstruction > 3) return "bad reconstruction";
  if (p.riemann_solver < 0 || p.riemann_solver > 2) return "bad riemann_solver";
  if (p.time_stepping < 0 || p.time_stepping > 1) return "bad time_stepping";
  if (p.gravity_mode < 0 || p.gravity_mode > 2) return "bad gravity mode";
  if (p.thermal_conductivity_mode < 0 || p.thermal_conductivity_mode > 1) return "bad conductivity_mode";
  if (p.bctc_ymin < 0 || p.bctc_ymin > 2 || p.bctc_ymax < 0 || p.bctc_ymax > 2) return "bad thermal bc";
  if (p.viscosity_mode != 0) return "bad viscosity_mode";
  if (p.analytical_gravity_mode != 0) return "bad analytical_mode";
  return nullptr;
}

}  // namespace fv2d
