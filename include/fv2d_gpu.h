/*
 * fv2d_gpu.h -- C-ABI of the GB300 (sm_103a) explicit hydro step,
 * libfv2d_gpu.so.
 *
 * The reference has no FFI: its per-step boundary is the in-binary C++
 * functor API called from main.cpp.  Each entry point below replaces one of
 * those calls and keeps its argument meaning:
 *
 *   fv2d_create / fv2d_destroy      <- readInifile + View allocation
 *                                      (SimInfo.h:529-568, main.cpp:33-34)
 *                                      and the functor constructors
 *                                      (Update.h:50-56, ComputeDt.h:15)
 *   fv2d_init_problem               <- InitFunctor::init + primToCons
 *                                      (Init.h:310-358, main.cpp:58)
 *   fv2d_set_prim / fv2d_get_prim   <- loadSnapshot copy-in / saveSolution
 *                                      copy-out (IOManager.h:358-379,
 *                                      IOManager.h:244-262)
 *   fv2d_compute_dt                 <- ComputeDtFunctor::computeDt
 *                                      (ComputeDt.h:18-65)
 *   fv2d_update                     <- UpdateFunctor::update + consToPrim +
 *                                      checkNegatives (Update.h:193-222,
 *                                      SimInfo.h:576-646, main.cpp:79-81)
 *   fv2d_get_counters               <- the three counts printed by
 *                                      checkNegatives (SimInfo.h:637-645)
 *   fv2d_advance                    <- the whole main.cpp:62-84 loop body,
 *                                      iterated on the device without host
 *                                      round trips (stops at tend or at a
 *                                      snapshot time)
 *
 * Conventions: every function returns an FV2D_* status (fv2d_types.h); no
 * C++ exception crosses the ABI.  A context is not thread-safe; separate
 * contexts are independent.  Host arrays use the interior row-major layout
 * described in fv2d_types.h.  All work is queued on the context's stream;
 * functions that return host values synchronise that stream.
 */
#ifndef FV2D_GPU_H
#define FV2D_GPU_H

#include "fv2d_types.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fv2d_ctx fv2d_ctx;

/* Reference defaults (SimInfo.h:356-459, 529-552) exactly as the reference
 * holds them after reading an .ini that leaves them unset: real-valued
 * parameters pass through INIReader::GetFloat and are therefore
 * float-rounded (gamma0 = (float)(5/3), CFL = 0.8f, ...). */
void fv2d_params_default(fv2d_params *p);

/* Validates p, selects device `device` (-1: current), allocates the state
 * (two primitive buffers, the conservative buffer, RK2 stage buffer when
 * time_stepping == RK2) and builds the TMA descriptors. */
int fv2d_create(const fv2d_params *p, int device, fv2d_ctx **out);
int fv2d_destroy(fv2d_ctx *ctx);

/* Work is queued on this stream (a cudaStream_t; NULL = the context's own
 * stream). */
int fv2d_set_stream(fv2d_ctx *ctx, void *stream);

/* Initial condition `problem` (FV2D_PB_*) computed on the host in binary64,
 * uploaded, then boundary fill, primToCons and the dt reduction. */
int fv2d_init_problem(fv2d_ctx *ctx, int problem);

/* Interior primitive state (Ny x Nx x {rho,u,v,p}) from / to host memory.
 * set_prim behaves like a restart: boundary fill, primToCons, dt reduction;
 * it returns once q_host has been consumed.  Page-locked host memory is read
 * by the set-up kernel directly over the host link (no staging copy). */
int fv2d_set_prim(fv2d_ctx *ctx, const double *q_host);
int fv2d_get_prim(fv2d_ctx *ctx, double *q_host);

/* Input prefetch (no reference counterpart): starts copying the page-locked
 * host array q_host (Ny x Nx x 4 doubles) into the context's staging buffer
 * on a copy stream of its own and returns at once; the state is not changed.
 * The copy overlaps the work already queued on the context's stream (a step
 * in flight reads the host link's other direction or not at all), so a
 * caller that feeds each step a new input from host memory can read the next
 * input during the current step.  The next fv2d_set_prim(ctx, q_host) with
 * the same pointer then builds the state from the staging buffer instead of
 * reading the host link.  q_host must not change between the two calls.  Any
 * other use of the staging buffer in between (fv2d_set_prim with another
 * pageable array, fv2d_set_prim_device, fv2d_init_problem, fv2d_get_prim
 * other than of the host mirror, fv2d_get_cons) waits for the copy and drops
 * it; fv2d_set_prim then reads q_host again.  FV2D_ERR_INVALID for pageable
 * memory. */
int fv2d_prefetch_prim(fv2d_ctx *ctx, const double *q_host);

/* Host mirror (no reference counterpart): registers a page-locked, 16-byte
 * aligned host array of Ny x Nx x 4 doubles that every fv2d_update also
 * writes the new interior primitives into, from the step kernel itself while
 * it computes (the transfer overlaps the step instead of following it).
 * fv2d_get_prim on that same pointer then only waits for the step.  The
 * device-driven loops (fv2d_advance, fv2d_run_async) do not write it.  NULL
 * detaches; the array must stay valid while registered. */
int fv2d_set_host_mirror(fv2d_ctx *ctx, double *q_host);
/* Interior conservative state (rho, rho u, rho v, E). */
int fv2d_get_cons(fv2d_ctx *ctx, double *u_host);

/* Same as set_prim / get_prim with device-resident interleaved arrays.
 * set_prim_device is ordered on the context's stream and returns before the
 * copy has run: q_dev must not change until work on that stream after the
 * call (or a synchronisation) has completed.  get_prim_device returns with the
 * copy complete. */
int fv2d_set_prim_device(fv2d_ctx *ctx, const double *q_dev);
int fv2d_get_prim_device(fv2d_ctx *ctx, double *q_dev);

/* ComputeDtFunctor::computeDt of the current primitive state:
 * dt = CFL / max(inv_dt_hyp, inv_dt_tc, inv_dt_visc).  Any output pointer
 * may be NULL.  The reductions are folded into the previous update (or the
 * set_prim / init_problem pass), so this call only reads them back. */
int fv2d_compute_dt(fv2d_ctx *ctx, double *dt, double *inv_dt_hyp, double *inv_dt_tc, double *inv_dt_visc);

/* One reference iteration body with the caller's dt: update(Q, U, dt),
 * consToPrim(U, Q), checkNegatives(Q).  Asynchronous. */
int fv2d_update(fv2d_ctx *ctx, double dt);

/* {negative density, negative pressure, NaN count} found by the
 * checkNegatives of the last update.  Synchronises. */
int fv2d_get_counters(fv2d_ctx *ctx, uint64_t out[3]);

/* Error bits set by the context's kernels since it was created (no reference
 * counterpart): 1 = a bounded TMA wait gave up, 2 = an index out of range
 * (only the bounds-check build, -DFV2D_BOUNDS_CHECK, tests for these). */
int fv2d_get_device_errors(fv2d_ctx *ctx, int *bits);

/* Device-driven main loop.  Runs at most max_steps iterations of
 *   while (t + epsilon < tend) { [stop if t + epsilon > next_save];
 *                                dt = computeDt; update; t += dt; }
 * entirely on the GPU (CUDA-graph replays of the fused step), then
 * synchronises.  next_save < 0 disables the snapshot stop.  When
 * skip_first_save_check is non-zero the snapshot test is skipped for the first
 * iteration (the caller just wrote that snapshot).  On return *t, *steps_done
 * and *status (FV2D_RUN_*) describe where the loop stopped. */
enum { FV2D_RUN_STEPS = 0, FV2D_RUN_DONE = 1, FV2D_RUN_SAVE = 2, FV2D_RUN_NUMERIC = 3 };
int fv2d_advance(fv2d_ctx *ctx, int max_steps, double tend, double next_save, int skip_first_save_check,
                 double *t, int *steps_done, int *status);

/* Queues n device-driven iterations on the context's stream and returns
 * without synchronising: each iteration computes its dt on the device from
 * the previous state (ComputeDt.h:18-65), updates (Update.h:193-222,
 * SimInfo.h:576-646) and advances t (main.cpp:83).  No tend or snapshot stop;
 * a non-finite or non-positive dt stops the remaining iterations.  Exactly n
 * step launches (2n with RK2) plus one control launch are queued. */
int fv2d_run_async(fv2d_ctx *ctx, int n);

/* Simulation clock kept on the device (t after the last committed update,
 * iteration count).  set_time resets both (e.g. after a restart). */
int fv2d_get_time(fv2d_ctx *ctx, double *t, int *iteration);
int fv2d_set_time(fv2d_ctx *ctx, double t, int iteration);

/* Per-iteration records of the last fv2d_advance / fv2d_run_async call (the
 * first 4096 iterations): 6 doubles per iteration, {t before the update, dt,
 * inv_dt_hyp of the state dt was computed from, negative-density count,
 * negative-pressure count, NaN count} -- what main.cpp:60-70 and
 * checkNegatives (SimInfo.h:637-645) print.  *count receives the number of
 * records written (at most max_records). */
int fv2d_get_step_log(fv2d_ctx *ctx, double *records, int max_records, int *count);

/* Human-readable message of the last failure on this context (never NULL). */
const char *fv2d_last_error(fv2d_ctx *ctx);

/* Static description of the compiled kernels: writes a short text (tile
 * shape, threads per block, architecture) into buf. */
int fv2d_build_info(char *buf, int len);

/* Allocation-free CFL time step.  No counterpart in the reference: it exists
 * for callers that cannot call cudaMalloc -- code whose device memory belongs
 * to another allocator (a framework pool that must account for every byte, or
 * a process that reserved all device memory up front) and loops that cannot
 * afford the device-wide synchronisation an allocation may cause.
 *
 * Takes a caller-owned device array q_dev of interleaved interior primitives
 * (Ny x Nx x {rho,u,v,p}, the layout of fv2d_set_prim_device) and writes
 * {dt, inv_dt_hyp, inv_dt_tc, inv_dt_visc} to the caller-owned device array
 * out_dev (4 doubles), queued on `stream` (a cudaStream_t, NULL = default
 * stream); the result equals fv2d_compute_dt's on the same state bit for bit
 * (NaN cells included: like fv2d_compute_dt it skips them).
 * It allocates nothing: its only scratch is a fixed array inside the library
 * (32 KB + 256 B on every GPU that loads the library, held until exit), which
 * limits the grid to FV2D_NOALLOC_MAX_CELLS cells; larger grids return
 * FV2D_ERR_SIZE before any GPU work.  The first call on a device loads the
 * library's device code there if nothing has yet (CUDA loads modules lazily;
 * that load may allocate and synchronise) and looks up the array's device
 * address with that device current; later calls allocate nothing.  Make that
 * first call before the loop that must not allocate and before any stream
 * capture, and do not call it on a device after cudaDeviceReset.  All calls
 * share the array: calls whose work overlaps on the GPU (other streams, other
 * host threads) race -- serialise them. */
#define FV2D_NOALLOC_CELLS_PER_BLOCK 4096
#define FV2D_NOALLOC_MAX_CELLS (4096 * 4096)
int fv2d_compute_dt_noalloc(const fv2d_params *p, const double *q_dev, double *out_dev, void *stream);

/* ------------------------------------------------------------------------
 * Measurement and test hooks.  Not part of the drop-in interface: nothing in
 * the step or the service calls them; the benchmark and the tests use them to
 * state the FP64 roofline and to check the device arithmetic and the bounded
 * waits on the GPU that runs the library.
 * ------------------------------------------------------------------------ */

/* Measurement hook: measured binary64 fused multiply-add throughput of
 * `device` in GFLOP/s (2 flops per DFMA), from a dependent-chain-free DFMA
 * loop timed with CUDA events.  Used to state the FP64 roofline of the step
 * kernel. */
int fv2d_probe_fp64_peak(int device, double *gflops);

/* Test hook: self-test of the step kernel's binary64 arithmetic on the integer pipes:
 * op 0 = division, 1 = square root, 2 = comparisons, 3 = fmax / fmin,
 * 4 = scalings by powers of two, 5 = multiplication.  Evaluates n generated operand sets
 * (random significands, arbitrary bit patterns, near-tie and exact cases,
 * extreme exponents) with both the integer routine and the hardware
 * instruction and counts results whose bits differ (NaNs compare equal).
 * example receives {a, b, integer result} of the first mismatch. */
int fv2d_selftest_arith(int op, uint64_t n, uint64_t seed, uint64_t *mismatches, double example[3]);

/* Test hook: self-test of the device-side wait guard (no reference counterpart): one
 * thread waits, with the step kernel's bounded wait and an iteration limit of
 * `limit` (1 .. 2^20), on a barrier that is never completed.  *timed_out
 * receives the error bits the wait sets (DEVERR_TMA_TIMEOUT = 1) instead of
 * hanging; the context stays usable afterwards. */
int fv2d_selftest_wait_timeout(uint32_t limit, int *timed_out);

/* sizeof(fv2d_params) as compiled into the library. */
size_t fv2d_params_size(void);

#ifdef __cplusplus
}
#endif
#endif /* FV2D_GPU_H */
