/*
 * fv2d_serve.h -- batched FP32 service of libfv2d_gpu.so: many independent
 * fv2d simulations of different sizes admitted as they arrive and advanced
 * together on one GB300.
 *
 * No counterpart in the reference (which runs one simulation per process,
 * main.cpp:13-101); each simulation follows the reference's step
 * (ComputeDt.h:18-65, Update.h:93-222, SimInfo.h:576-646) -- every Riemann
 * solver, reconstruction (and the MUSCL-Hancock extension), time stepping,
 * gravity, conduction and viscosity setting of fv2d_params, on any Nx x Ny
 * grid -- in binary32 storage and flux arithmetic, with the simulation clock,
 * dt, the conservation sums and (for low-Mach requests) the internal-energy
 * recovery E - rho|u|^2/2 in binary64.  The state is stored as its offset
 * from a per-request background density and total energy (the medians of the
 * initial condition), which keeps more digits where the flow stays near it.
 *
 * Serving model:
 *   - fv2d_server_submit queues a request; a worker thread admits queued
 *     requests (first in, first out, smaller ones may pass a request that
 *     does not fit) while the HBM budget and the simulation table allow;
 *   - every admitted state stays resident in HBM until it completes;
 *   - requests fall into three kernel families: plain (HLL / HLLC, PCM /
 *     PLM, constant gravity), diffusive (the same with constant conduction
 *     and / or viscosity) and extended (FSLP, MUSCL-Hancock, analytical
 *     gravity, B02 conductivity, the y-boundary conduction modes, the
 *     well-balanced y flux);
 *   - all admitted simulations advance together: per lane (grid-size bucket
 *     of one kernel family) one persistent kernel launch per stage walks a
 *     (simulation, tile) work list, each simulation reduces its own dt; an
 *     SSP-RK2 step takes two launches; a CUDA graph replays several launches
 *     between admissions and retirements, the lanes as parallel branches;
 *   - the kernel configuration (tile shape or column strip, threads per
 *     CTA, halo staging) is chosen per family by an autotuner at start-up,
 *     one for all of the family's buckets (or fixed defaults per bucket).
 * A simulation's result does not depend on what else was in the batch.
 *
 * Failures:
 *   - a request whose dt guard trips completes with FV2D_ERR_NUMERIC; the
 *     others are not affected;
 *   - a request whose final state cannot be copied to host memory completes
 *     with FV2D_ERR_NOMEM and keeps no state;
 *   - if a CUDA call of the worker fails (the CUDA context is then unusable),
 *     or host memory runs out while the worker changes its tables, the
 *     service stops: every resident and queued request completes with
 *     FV2D_ERR_CUDA (resp. FV2D_ERR_NOMEM), fv2d_server_submit returns
 *     FV2D_ERR_STATE, fv2d_server_drain returns that code at once and
 *     fv2d_server_last_error says what failed.  Device memory is released by
 *     fv2d_server_destroy.
 */
#ifndef FV2D_SERVE_H
#define FV2D_SERVE_H

#include "fv2d_types.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fv2d_server fv2d_server;

typedef struct fv2d_server_config {
  uint32_t struct_size;
  int32_t device;           /* CUDA device */
  double budget_bytes;      /* HBM budget for simulation states (admission control) */
  int32_t max_sims;         /* simulation table capacity (<= 16384) */
  int32_t autotune;         /* 1: time the kernel configurations per family at start-up */
  int32_t steps_per_replay; /* 0: adaptive (about 3 ms of work per graph replay) */
  int32_t tile_config;      /* 0: defaults or autotuned; k > 0: configuration k - 1 for every bucket of the
                               kernel families it serves (the others keep their defaults) */
  double active_cells;      /* 0: every admitted request advances at every step.  > 0: shortest remaining
                               work first -- the requests with the fewest remaining cell-updates advance,
                               about this many cells per step (at least one request); the others stay
                               resident in HBM until they rank among them */
  int32_t single_launch;    /* 0: one work list and one launch per lane (grid-size bucket x kernel family), the
                               lanes as parallel graph branches.  1: every request of a kernel family in one
                               work list, advanced by one persistent launch per step with one configuration
                               (the one chosen for the largest grids) */
  int32_t band_rows;        /* 0: the march kernels' rows per work item are chosen per lane at every work-list
                               rebuild (to fill whole waves of the launch's resident warps); 8..64: that many */
} fv2d_server_config;

typedef struct fv2d_request {
  uint32_t struct_size;
  int32_t problem;   /* FV2D_PB_* initial condition */
  fv2d_params params;/* any valid parameter block with 16 <= Nx, Ny <= 8192 */
  int32_t max_steps; /* stop after this many steps */
  int32_t lowmach;   /* 1: recover the pressure from E - rho|u|^2/2 in binary64 where it cancels */
  double tend;       /* also stop once t + epsilon >= tend (<= 0: no time limit) */
} fv2d_request;

typedef struct fv2d_result {
  int64_t id;
  int32_t status;    /* FV2D_OK; FV2D_ERR_NUMERIC when the NaN / dt guard stopped it; FV2D_ERR_CUDA when a
                        tile copy outlived its bounded wait (fv2d_server_set_tile_wait_limit) */
  int32_t steps;     /* steps taken */
  double t;          /* simulation time reached (binary64 clock) */
  double submit_s, admit_s, done_s;  /* server clock, seconds since fv2d_server_create */
  double cons0[4];   /* sum over cells of (rho, rho u, rho v, E) * dx * dy at admission, */
  double cons1[4];   /* and at completion: compensated binary64 sums of the binary32 state */
  uint64_t negatives;/* cells reset by the negative density/pressure guard */
  int32_t Nx, Ny;
  int32_t bucket;    /* grid-size bucket (0..3) */
  int32_t lane;      /* bucket, + 4 when the diffusive kernel family ran it, + 8 for the extended one */
} fv2d_result;

typedef struct fv2d_server_stats {
  int64_t submitted, admitted, completed, failed;
  int32_t active, queued;
  double cell_updates;   /* total cell-updates performed */
  double busy_s;         /* wall time with at least one active simulation */
  double bytes_in_use;   /* HBM held by resident states */
  double bytes_reserved; /* HBM reserved by the state arena */
  int32_t bucket_cfg[4]; /* plain-family configuration index per bucket (see fv2d_server_config_name) */
  int32_t replays;       /* graph replays launched */
  int32_t ext_cfg;       /* extended-family configuration index */
  int32_t diff_cfg[4];   /* diffusive-family configuration index per bucket */
} fv2d_server_stats;

int fv2d_server_create(const fv2d_server_config *cfg, fv2d_server **out);
int fv2d_server_destroy(fv2d_server *s);

/* The checks fv2d_server_submit makes on a request's own fields, without a
 * server or a GPU: FV2D_OK, or FV2D_ERR_UNSUPPORTED with the reason written
 * into buf (len bytes at most, NUL-terminated; "" when accepted). */
int fv2d_server_check_request(const fv2d_request *req, char *buf, int len);

/* Queue a request; returns its id.  FV2D_ERR_UNSUPPORTED (see
 * fv2d_server_check_request), FV2D_ERR_SIZE when its state can never fit the
 * budget, FV2D_ERR_STATE once the service has stopped.  Thread-safe. */
int fv2d_server_submit(fv2d_server *s, const fv2d_request *req, int64_t *id);

/* Results completed since the last poll (at most max); *n receives the count. */
int fv2d_server_poll(fv2d_server *s, fv2d_result *out, int max, int *n);

/* Block until nothing is queued or running: FV2D_OK; FV2D_ERR_STATE when
 * timeout_s (>= 0, may be infinite) elapses first; the stopping code when the
 * service has stopped (see Failures above). */
int fv2d_server_drain(fv2d_server *s, double timeout_s);

/* Final primitive state of a completed request (Ny x Nx x {rho,u,v,p}, binary64
 * values of the binary32 state), until fv2d_server_release. */
int fv2d_server_get_prim(fv2d_server *s, int64_t id, double *q_host);
int fv2d_server_release(fv2d_server *s, int64_t id);

int fv2d_server_get_stats(fv2d_server *s, fv2d_server_stats *out);

/* Why the service stopped ("" while it runs), copied into buf (len bytes at
 * most, NUL-terminated).  Thread-safe. */
int fv2d_server_last_error(fv2d_server *s, char *buf, int len);

/* Test hook for the failure path above, with no GPU fault: the worker stops
 * after its current replay as if a CUDA call had failed. */
int fv2d_server_inject_fault(fv2d_server *s);

/* Test hook for the bounded tile-copy wait, with no GPU fault: the served
 * kernels that stage tiles by TMA poll a copy's barrier at most `polls` times
 * (default 2^24; 0 = not at all) before they fail the simulation the tile
 * belongs to (its result completes with FV2D_ERR_CUDA) and wait once more,
 * bounded, for the copy to land before the tile buffer is used again.  A copy
 * that outlives that second wait stops the service as a failed CUDA call
 * does.  Applied by the worker before its next replay. */
int fv2d_server_set_tile_wait_limit(fv2d_server *s, uint32_t polls);

/* Name of kernel configuration `index` ("32x16/256/tma", "28/32x20/march", "60/32x16/march2", ...); NULL if
 * none.  The names of the march kernels read <strip columns>/<threads per CTA>x<CTAs per SM>/<kernel>. */
const char *fv2d_server_config_name(int index);

/* Kernel families configuration `index` serves, as a bit mask: 1 plain (HLL / HLLC, PCM / PLM, constant
 * gravity), 2 diffusive (the same with constant conduction and / or viscosity), 4 extended (FSLP,
 * MUSCL-Hancock, analytical gravity, B02 conductivity, the y-boundary conduction modes, the well-balanced y
 * flux); -1 if there is no such configuration.  Needs no GPU. */
int fv2d_server_config_families(int index);

#ifdef __cplusplus
}
#endif
#endif /* FV2D_SERVE_H */
