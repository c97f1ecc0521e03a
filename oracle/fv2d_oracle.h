/*
 * fv2d_oracle.h -- TEST INFRASTRUCTURE, not part of the product.
 *
 * CPU FP64 restatement of the reference's explicit hydro step
 * (mdelorme/fv2d: States.h, RiemannSolvers.h, Gravity.h,
 * BoundaryConditions.h, Update.h, ThermalConduction.h, Viscosity.h,
 * ComputeDt.h, SimInfo.h:576-646, Init.h, main.cpp:62-84).  It keeps the
 * reference's pass structure (boundary fill -> slope arrays -> per-cell
 * update that solves every face twice -> thermal conduction -> viscosity ->
 * consToPrim -> checkNegatives, max-reduction for dt) and its exact order of
 * floating-point operations, compiled with -ffp-contract=off.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
 * load this library, and only as the oracle results are compared against or
 * as the timed CPU baseline; the product path never calls it.
 *
 * Pinning: the restatement is checked against (1) the reference's only
 * published known answers (README.md:86-89, the blast.ini dt log) and
 * (2) fixtures produced by compiling the reference's own hot-path headers
 * against a minimal serial stand-in for the Kokkos/inih entry points they use
 * (oracle/ref_check/), committed under tests/golden/.
 */
#ifndef FV2D_ORACLE_H
#define FV2D_ORACLE_H

#include "../include/fv2d_types.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fv2d_oracle fv2d_oracle;

/* Defaults of SimInfo.h:356-459 and SimInfo.h:529-552. */
void fv2d_oracle_params_default(fv2d_params *p);

int fv2d_oracle_create(const fv2d_params *p, fv2d_oracle **out);
void fv2d_oracle_destroy(fv2d_oracle *o);

/* Init.h:310-358: interior initial condition, then boundary fill, then
 * primToCons over the whole array (main.cpp:58). */
int fv2d_oracle_init_problem(fv2d_oracle *o, int problem);

/* Interior primitive state in/out (layout in fv2d_types.h). set_prim also
 * fills the ghosts and rebuilds U = primToCons(Q) like a restart
 * (IOManager.h:358-379 then main.cpp:58). */
int fv2d_oracle_set_prim(fv2d_oracle *o, const double *q);
int fv2d_oracle_get_prim(const fv2d_oracle *o, double *q);
int fv2d_oracle_get_cons(const fv2d_oracle *o, double *u);

/* ComputeDt.h:18-65.  out = {dt, inv_dt_hyp, inv_dt_tc, inv_dt_visc}. */
int fv2d_oracle_compute_dt(const fv2d_oracle *o, double out[4]);

/* One iteration body of main.cpp:79-81: update(Q, U, dt), consToPrim(U, Q),
 * checkNegatives(Q). */
int fv2d_oracle_update(fv2d_oracle *o, double dt);

/* Accuracy-floor hook (no counterpart in the reference): rounds every stored
 * conservative value (ghosts included) to binary32 as the offset U - bg[v]
 * from a constant background (bg may be NULL for zero), then rebuilds Q with
 * consToPrim and checkNegatives.  Called after each update, it gives a run in
 * binary64 arithmetic whose state is stored the way a binary32 service stores
 * it: the error that storage alone causes. */
int fv2d_oracle_round_cons_f32(fv2d_oracle *o, const double *bg);

/* Counters of the last checkNegatives: {negative density, negative
 * pressure, NaN count} (SimInfo.h:602-646). */
int fv2d_oracle_get_counters(const fv2d_oracle *o, uint64_t out[3]);

/* The main.cpp:62-84 loop without snapshots: while (t + eps < tend)
 * { dt = computeDt; update; t += dt } for at most max_steps iterations.
 * dts (may be NULL) receives every dt; returns the iteration count in *nsteps
 * and the final time in *t_io (which also carries the start time in). */
int fv2d_oracle_run(fv2d_oracle *o, double tend, int max_steps, double *t_io, int *nsteps, double *dts);

/* OpenMP thread count used by every pass (<= 0 keeps the runtime default). */
void fv2d_oracle_set_threads(int n);
int fv2d_oracle_get_threads(void);

/* Counter-based generator used by the seeded problems (H84, C91, KH_STEP):
 * SplitMix64 (Steele, Lea, Flood 2014) of (seed, cell, stream), 53-bit
 * uniform in [0, 1). */
double fv2d_oracle_uniform(int32_t seed, int64_t cell, int32_t stream);

#ifdef __cplusplus
}
#endif
#endif
