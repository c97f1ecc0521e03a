/*
 * fv2d_types.h -- plain-C parameter block and enumerations shared by the
 * GB300 hydro-step library (libfv2d_gpu.so), its C++ host driver and the
 * CPU oracle used by the tests.
 *
 * Every field mirrors one member of the reference's parameter structs and
 * keeps the reference's default (SimInfo.h:266-354 DeviceParams,
 * SimInfo.h:463-492 Params, defaults read in SimInfo.h:356-459 and
 * SimInfo.h:529-552).  Enumerator values follow the reference's enums
 * (SimInfo.h:26-97) so that integer codes coming from a reference-side
 * binding keep their meaning.
 *
 * Layout conventions at the boundary:
 *   - primitive / conservative cell arrays crossing the ABI are interior-only,
 *     row-major with j (y) outer, i (x) inner and the 4 fields fastest:
 *     q[((j * Nx) + i) * 4 + f], f in {rho, u, v, p} (or {rho, rho*u, rho*v, E}).
 *     This is the reference's Array(Nty, Ntx, 4) restricted to
 *     [jbeg, jend) x [ibeg, iend) (SimInfo.h:17, main.cpp:33-34).
 *   - all arithmetic is IEEE binary64 unless a function says otherwise.
 */
#ifndef FV2D_TYPES_H
#define FV2D_TYPES_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Field indices (SimInfo.h:32-39). */
enum { FV2D_IR = 0, FV2D_IU = 1, FV2D_IV = 2, FV2D_IP = 3, FV2D_IE = 3, FV2D_NFIELDS = 4 };

/* RiemannSolver (SimInfo.h:41-46). */
enum { FV2D_HLL = 0, FV2D_HLLC = 1, FV2D_FSLP = 2 };

/* BoundaryType (SimInfo.h:48-53). */
enum { FV2D_BC_ABSORBING = 0, FV2D_BC_REFLECTING = 1, FV2D_BC_PERIODIC = 2 };

/* TimeStepping (SimInfo.h:55-59). */
enum { FV2D_TS_EULER = 0, FV2D_TS_RK2 = 1 };

/* ReconstructionType (SimInfo.h:61-66).  FV2D_MUSCL_HANCOCK is an extension
 * with no reference counterpart: PLM face states advanced by the
 * characteristic-free half-step q -= dt/(2d) * A(q) dq before the Riemann
 * solve.  It is never selected by a reference .ini file. */
enum { FV2D_PCM = 0, FV2D_PCM_WB = 1, FV2D_PLM = 2, FV2D_MUSCL_HANCOCK = 3 };

/* ThermalConductivityMode (SimInfo.h:68-72). */
enum { FV2D_TCM_CONSTANT = 0, FV2D_TCM_B02 = 1 };

/* BCTC_Mode (SimInfo.h:75-80). */
enum { FV2D_BCTC_NONE = 0, FV2D_BCTC_FIXED_TEMPERATURE = 1, FV2D_BCTC_FIXED_GRADIENT = 2 };

/* ViscosityMode (SimInfo.h:82-85). */
enum { FV2D_VSC_CONSTANT = 0 };

/* GravityMode (SimInfo.h:87-92). */
enum { FV2D_GRAV_NONE = 0, FV2D_GRAV_CONSTANT = 1, FV2D_GRAV_ANALYTICAL = 2 };

/* AnalyticalGravityMode (SimInfo.h:94-97). */
enum { FV2D_AGM_HOT_BUBBLE = 0 };

/* InitType (Init.h:271-282) followed by problems with no reference
 * counterpart (the benchmark set-ups: a point-energy Sedov blast, a sharp
 * shear-layer Kelvin-Helmholtz with seeded noise and a hydrostatic
 * Rayleigh-Taylor). */
enum {
  FV2D_PB_SOD_X = 0,
  FV2D_PB_SOD_Y = 1,
  FV2D_PB_BLAST = 2,
  FV2D_PB_RAYLEIGH_TAYLOR = 3,
  FV2D_PB_DIFFUSION = 4,
  FV2D_PB_H84 = 5,
  FV2D_PB_C91 = 6,
  FV2D_PB_KELVIN_HELMHOLTZ = 7,
  FV2D_PB_GRESHO_VORTEX = 8,
  FV2D_PB_SEDOV = 100,
  FV2D_PB_KH_STEP = 101,
  FV2D_PB_RT_HYDROSTATIC = 102
};

/* Status codes returned by every entry point. */
enum {
  FV2D_OK = 0,
  FV2D_ERR_INVALID = 1,    /* bad argument or parameter combination */
  FV2D_ERR_CUDA = 2,       /* a CUDA runtime call failed */
  FV2D_ERR_NOMEM = 3,      /* device or host allocation failed */
  FV2D_ERR_STATE = 4,      /* call out of order (e.g. update before set_prim) */
  FV2D_ERR_NUMERIC = 5,    /* NaN or non-positive dt detected by the device guard */
  FV2D_ERR_UNSUPPORTED = 6, /* valid in the reference but not provided here */
  FV2D_ERR_SIZE = 7         /* input larger than a fixed-size limit of the entry point */
};

/* The full parameter block.  Fill with fv2d_params_default() and override.
 * struct_size must equal sizeof(fv2d_params); it lets a caller compiled
 * against an older header be rejected cleanly. */
typedef struct fv2d_params {
  uint32_t struct_size;

  /* [mesh] SimInfo.h:360-376 */
  int32_t Nx, Ny, Nghosts;
  double xmin, xmax, ymin, ymax;

  /* [run] / [solvers] SimInfo.h:378-389, 536-545 */
  double CFL;
  int32_t boundary_x, boundary_y;
  int32_t reconstruction;
  int32_t riemann_solver;
  int32_t time_stepping;
  double tend, save_freq;

  /* [physics] / [misc] SimInfo.h:392-399, 549-551 */
  double gamma0;
  double epsilon;
  double epsilon_reset_negative;
  int32_t well_balanced_flux_at_y_bc;
  double fslp_K;
  int32_t seed;
  int32_t log_frequency;

  /* [gravity] SimInfo.h:402-411, 444 */
  int32_t gravity_mode;
  int32_t analytical_gravity_mode;
  double gx, gy;
  double hot_bubble_g0;

  /* [thermal_conduction] SimInfo.h:414-427.  The B02 profile constants
   * (SimInfo.h:307-310) are never read from a file by the reference; they are
   * plain inputs here. */
  int32_t thermal_conductivity_active;
  int32_t thermal_conductivity_mode;
  double kappa;
  int32_t bctc_ymin, bctc_ymax;
  double bctc_ymin_value, bctc_ymax_value;
  double b02_ymid, b02_kappa1, b02_kappa2, b02_thickness;

  /* [viscosity] SimInfo.h:430-435 */
  int32_t viscosity_active;
  int32_t viscosity_mode;
  double mu;

  /* problem parameters: [polytrope] [H84] [C91] [kelvin_helmholtz]
   * [gresho_vortex] SimInfo.h:394-397, 438-458 */
  double m1, theta1, m2, theta2;
  double h84_pert, c91_pert;
  double kh_a, kh_amp, kh_P0, kh_rho_fac, kh_sigma, kh_uflow, kh_y1, kh_y2;
  double gresho_density, gresho_Mach;

  /* extension problems (no reference counterpart) */
  double sod_rho_left, sod_p_left, sod_rho_right, sod_p_right; /* SOD_X / SOD_Y states */
  double sedov_E0, sedov_r0, sedov_p_ambient, sedov_rho;
  double khs_rho_in, khs_rho_out, khs_u, khs_p0, khs_amp, khs_noise;
  double rt_rho_top, rt_rho_bottom, rt_p_interface, rt_y_interface, rt_amp;
} fv2d_params;

#ifdef __cplusplus
}
#endif
#endif /* FV2D_TYPES_H */
