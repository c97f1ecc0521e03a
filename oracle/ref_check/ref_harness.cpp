// ref_harness.cpp -- TEST INFRASTRUCTURE.  Drives the reference's own
// hot-path headers (compiled in place from the reference checkout, see
// oracle/ref_check/build.sh) through a small C API so that the tests can run
// them side by side with the oracle.  The call sequence restates main.cpp:
//   readInifile (main.cpp:21) -> InitFunctor::init or a restart-like
//   set_prim (IOManager.h:358-379) -> primToCons (main.cpp:58) ->
//   per iteration: computeDt (main.cpp:66), update + consToPrim +
//   checkNegatives (main.cpp:79-81).
#include "SimInfo.h"
#include "BoundaryConditions.h"
#include "ComputeDt.h"
#include "Init.h"
#include "Update.h"

#include <cstring>
#include <fstream>
#include <memory>

using namespace fv2d;

namespace {
struct RefSim {
  Params params;
  Array U, Q;
  std::unique_ptr<UpdateFunctor> update;
  std::unique_ptr<ComputeDtFunctor> cdt;
};
}  // namespace

extern "C" {

void *fv2d_ref_create(const char *ini_path) {
  try {
    auto *s = new RefSim();
    s->params = readInifile(ini_path);
    const auto &dp = s->params.device_params;
    s->U = Array("U", dp.Nty, dp.Ntx, Nfields);
    s->Q = Array("Q", dp.Nty, dp.Ntx, Nfields);
    s->update = std::make_unique<UpdateFunctor>(s->params);
    s->cdt = std::make_unique<ComputeDtFunctor>(s->params);
    return s;
  } catch (const std::exception &e) {
    std::cerr << "fv2d_ref_create: " << e.what() << std::endl;
    return nullptr;
  }
}

void fv2d_ref_destroy(void *h) { delete static_cast<RefSim *>(h); }

int fv2d_ref_dims(void *h, int *nx, int *ny) {
  auto *s = static_cast<RefSim *>(h);
  *nx = s->params.device_params.Nx;
  *ny = s->params.device_params.Ny;
  return 0;
}

// The effective real-valued parameters after the reference's ini reading.
int fv2d_ref_param(void *h, const char *name, double *out) {
  auto *s = static_cast<RefSim *>(h);
  const auto &d = s->params.device_params;
  std::string n(name);
  if (n == "gamma0") *out = d.gamma0;
  else if (n == "CFL") *out = d.CFL;
  else if (n == "epsilon") *out = d.epsilon;
  else if (n == "gx") *out = d.gx;
  else if (n == "gy") *out = d.gy;
  else if (n == "kappa") *out = d.kappa;
  else if (n == "mu") *out = d.mu;
  else if (n == "dx") *out = d.dx;
  else if (n == "dy") *out = d.dy;
  else if (n == "tend") *out = s->params.tend;
  else if (n == "save_freq") *out = s->params.save_freq;
  else if (n == "epsilon_reset_negative") *out = s->params.epsilon_reset_negative;
  else if (n == "fslp_K") *out = d.fslp_K;
  else return 1;
  return 0;
}

// Reader::outputValues of the parsed .ini (SimInfo.h:224-262).
int fv2d_ref_echo(void *h, const char *out_path) {
  auto *s = static_cast<RefSim *>(h);
  std::ofstream out(out_path);
  s->params.reader.outputValues(out);
  return out ? 0 : 1;
}

// Every DeviceParams / Params value the C-ABI parameter block mirrors, in a
// fixed order (doubles; integers and enums converted).
int fv2d_ref_dump(void *h, double *out, int n) {
  auto *s = static_cast<RefSim *>(h);
  const auto &d = s->params.device_params;
  const auto &P = s->params;
  const double v[] = {(double)d.Nx, (double)d.Ny, (double)d.Ng, d.xmin, d.xmax, d.ymin, d.ymax, d.CFL,
                      (double)d.boundary_x, (double)d.boundary_y, (double)d.reconstruction, (double)d.riemann_solver,
                      (double)P.time_stepping, P.tend, P.save_freq, d.gamma0, d.epsilon, P.epsilon_reset_negative,
                      (double)d.well_balanced_flux_at_y_bc, d.fslp_K, (double)P.seed, (double)P.log_frequency,
                      (double)d.gravity_mode, (double)d.analytical_gravity_mode, d.gx, d.gy, d.hot_bubble_g0,
                      (double)d.thermal_conductivity_active, (double)d.thermal_conductivity_mode, d.kappa,
                      (double)d.bctc_ymin, (double)d.bctc_ymax, d.bctc_ymin_value, d.bctc_ymax_value,
                      (double)d.viscosity_active, (double)d.viscosity_mode, d.mu, d.m1, d.theta1, d.m2, d.theta2,
                      d.h84_pert, d.c91_pert, d.kh_a, d.kh_amp, d.kh_P0, d.kh_rho_fac, d.kh_sigma, d.kh_uflow, d.kh_y1,
                      d.kh_y2, d.gresho_density, d.gresho_Mach};
  const int m = (int)(sizeof(v) / sizeof(v[0]));
  for (int k = 0; k < m && k < n; ++k) out[k] = v[k];
  return m;
}

int fv2d_ref_init(void *h) {
  auto *s = static_cast<RefSim *>(h);
  try {
    InitFunctor init(s->params);
    init.init(s->Q);
    primToCons(s->Q, s->U, s->params);
  } catch (const std::exception &e) {
    std::cerr << "fv2d_ref_init: " << e.what() << std::endl;
    return 1;
  }
  return 0;
}

int fv2d_ref_set_prim(void *h, const double *q) {
  auto *s = static_cast<RefSim *>(h);
  const auto &d = s->params.device_params;
  for (int j = 0; j < d.Ny; ++j)
    for (int i = 0; i < d.Nx; ++i)
      for (int v = 0; v < Nfields; ++v) s->Q(j + d.jbeg, i + d.ibeg, v) = q[((size_t)j * d.Nx + i) * 4 + v];
  BoundaryManager bc(s->params);
  bc.fillBoundaries(s->Q);
  primToCons(s->Q, s->U, s->params);
  return 0;
}

static int get_arr(RefSim *s, const Array &A, double *q) {
  const auto &d = s->params.device_params;
  for (int j = 0; j < d.Ny; ++j)
    for (int i = 0; i < d.Nx; ++i)
      for (int v = 0; v < Nfields; ++v) q[((size_t)j * d.Nx + i) * 4 + v] = A(j + d.jbeg, i + d.ibeg, v);
  return 0;
}
int fv2d_ref_get_prim(void *h, double *q) { return get_arr(static_cast<RefSim *>(h), static_cast<RefSim *>(h)->Q, q); }
int fv2d_ref_get_cons(void *h, double *u) { return get_arr(static_cast<RefSim *>(h), static_cast<RefSim *>(h)->U, u); }

double fv2d_ref_compute_dt(void *h, int diag) {
  auto *s = static_cast<RefSim *>(h);
  return s->cdt->computeDt(s->Q, 0.0, 0.0, diag != 0);
}

int fv2d_ref_update(void *h, double dt) {
  auto *s = static_cast<RefSim *>(h);
  s->update->update(s->Q, s->U, dt);
  consToPrim(s->U, s->Q, s->params);
  checkNegatives(s->Q, s->params);
  return 0;
}

}  // extern "C"
