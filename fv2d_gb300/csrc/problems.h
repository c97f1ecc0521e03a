// problems.h -- host-side parameter defaults, initial conditions and
// position-only tables of the plain path (see problems.cpp).
#pragma once

#include <stdint.h>

#include "../../include/fv2d_types.h"

namespace fv2d {

void params_default(fv2d_params *p);
const char *validate(const fv2d_params &p);  // nullptr when valid
bool problem_valid(int problem);
float analytical_gravity_row(const fv2d_params &p, int j);
void kappa_row(const fv2d_params &p, int j, double out[4]);
void parabolic_inv_dt(const fv2d_params &p, double *inv_tc, double *inv_visc);

}  // namespace fv2d
