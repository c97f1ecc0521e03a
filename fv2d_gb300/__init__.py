"""fv2d_gb300 -- GB300-native (sm_103a) explicit finite-volume hydro step of
mdelorme/fv2d, behind the C-ABI declared in include/fv2d_gpu.h.

This module is a thin ctypes binding of that ABI, shaped like the
reference's per-step functor calls (UpdateFunctor::update,
ComputeDtFunctor::computeDt, consToPrim/checkNegatives, InitFunctor::init).
Every call goes through the compiled library fv2d_gb300/lib/libfv2d_gpu.so;
there is no CPU fallback: if the library is missing, loading raises.
"""
import ctypes as C
import os

import numpy as np

from ._abi import (  # noqa: F401  (re-exported enums)
    Params, PROBLEMS, ERROR_NAMES, ERR_SIZE, as_float32,
    HLL, HLLC, FSLP, BC_ABSORBING, BC_REFLECTING, BC_PERIODIC, TS_EULER, TS_RK2,
    PCM, PCM_WB, PLM, MUSCL_HANCOCK, GRAV_NONE, GRAV_CONSTANT, GRAV_ANALYTICAL,
    BCTC_NONE, BCTC_FIXED_TEMPERATURE, BCTC_FIXED_GRADIENT, TCM_CONSTANT, TCM_B02,
)

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "lib", "libfv2d_gpu.so")

RUN_STEPS, RUN_DONE, RUN_SAVE, RUN_NUMERIC = 0, 1, 2, 3

_dp = C.POINTER(C.c_double)
_lib = None


class Fv2dError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"fv2d error {ERROR_NAMES.get(code, code)}: {msg}")
        self.code = code


def lib():
    """The loaded C-ABI library (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -m fv2d_gb300.build` "
                               "(no CPU fallback exists)")
        L = C.CDLL(LIB_PATH)
        vp = C.c_void_p
        L.fv2d_params_default.argtypes = [C.POINTER(Params)]
        L.fv2d_params_default.restype = None
        L.fv2d_params_size.restype = C.c_size_t
        L.fv2d_create.argtypes = [C.POINTER(Params), C.c_int, C.POINTER(vp)]
        L.fv2d_destroy.argtypes = [vp]
        L.fv2d_set_stream.argtypes = [vp, vp]
        L.fv2d_init_problem.argtypes = [vp, C.c_int]
        L.fv2d_set_prim.argtypes = [vp, _dp]
        L.fv2d_prefetch_prim.argtypes = [vp, vp]
        L.fv2d_get_prim.argtypes = [vp, _dp]
        L.fv2d_get_cons.argtypes = [vp, _dp]
        L.fv2d_set_prim_device.argtypes = [vp, vp]
        L.fv2d_get_prim_device.argtypes = [vp, vp]
        L.fv2d_set_host_mirror.argtypes = [vp, vp]
        L.fv2d_compute_dt.argtypes = [vp, _dp, _dp, _dp, _dp]
        L.fv2d_update.argtypes = [vp, C.c_double]
        L.fv2d_get_counters.argtypes = [vp, C.POINTER(C.c_uint64)]
        L.fv2d_get_device_errors.argtypes = [vp, C.POINTER(C.c_int)]
        L.fv2d_advance.argtypes = [vp, C.c_int, C.c_double, C.c_double, C.c_int, _dp,
                                   C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.fv2d_get_time.argtypes = [vp, _dp, C.POINTER(C.c_int)]
        L.fv2d_set_time.argtypes = [vp, C.c_double, C.c_int]
        L.fv2d_get_step_log.argtypes = [vp, _dp, C.c_int, C.POINTER(C.c_int)]
        L.fv2d_last_error.argtypes = [vp]
        L.fv2d_last_error.restype = C.c_char_p
        L.fv2d_build_info.argtypes = [C.c_char_p, C.c_int]
        L.fv2d_run_async.argtypes = [vp, C.c_int]
        L.fv2d_probe_fp64_peak.argtypes = [C.c_int, _dp]
        L.fv2d_compute_dt_noalloc.argtypes = [C.POINTER(Params), vp, vp, vp]
        L.fv2d_selftest_arith.argtypes = [C.c_int, C.c_uint64, C.c_uint64, C.POINTER(C.c_uint64), _dp]
        L.fv2d_selftest_wait_timeout.argtypes = [C.c_uint32, C.POINTER(C.c_int)]
        _lib = L
    return _lib


def default_params(**overrides):
    """The reference's effective defaults (float-rounded like its .ini
    reader), with overrides.  Real-valued overrides are taken as given; use
    as_float32() to mimic values read from an .ini file."""
    p = Params()
    lib().fv2d_params_default(C.byref(p))
    return p.update(**overrides)


def build_info():
    buf = C.create_string_buffer(256)
    lib().fv2d_build_info(buf, 256)
    return buf.value.decode()


def probe_fp64_peak(device=0):
    """Measured binary64 FMA throughput in GFLOP/s."""
    g = C.c_double()
    rc = lib().fv2d_probe_fp64_peak(device, C.byref(g))
    if rc != 0:
        raise Fv2dError(rc, "fp64 probe failed")
    return g.value


def selftest_wait_timeout(limit=1000):
    """Error bits set by a bounded device wait on a barrier that is never
    completed (1 = timed out and returned)."""
    flag = C.c_int()
    rc = lib().fv2d_selftest_wait_timeout(int(limit), C.byref(flag))
    if rc != 0:
        raise Fv2dError(rc, "wait self-test failed to run")
    return flag.value


def selftest_arith(op, n, seed=1):
    """Bit-for-bit check of the integer-pipe binary64 routines against the
    hardware on n generated operand sets: op 0 division, 1 square root,
    2 comparisons, 3 fmax / fmin, 4 power-of-two scalings, 5 multiplication;
    returns
    (mismatches, first mismatching {a, b, result})."""
    bad = C.c_uint64()
    ex = (C.c_double * 3)()
    rc = lib().fv2d_selftest_arith(int(op), int(n), int(seed), C.byref(bad), ex)
    if rc != 0:
        raise Fv2dError(rc, "self-test failed to run")
    return bad.value, list(ex)


NOALLOC_MAX_CELLS = 4096 * 4096


def compute_dt_noalloc(params, q_dev_ptr, out_dev_ptr, stream_ptr=0):
    """Allocation-free CFL dt of a device array of interleaved interior
    primitives (for callers that cannot allocate device memory); writes
    {dt, inv_dt_hyp, inv_dt_tc, inv_dt_visc} to the device array at
    out_dev_ptr.  Returns the FV2D status code."""
    return lib().fv2d_compute_dt_noalloc(C.byref(params), C.c_void_p(q_dev_ptr), C.c_void_p(out_dev_ptr),
                                         C.c_void_p(stream_ptr))


def _ptr(a):
    return a.ctypes.data_as(_dp)


class Simulation:
    """One simulation on one GPU (an fv2d_ctx)."""

    def __init__(self, params, device=0):
        self._lib = lib()
        self.params = params.copy()
        self.h = C.c_void_p()
        rc = self._lib.fv2d_create(C.byref(self.params), device, C.byref(self.h))
        if rc != 0:
            raise Fv2dError(rc, self._lib.fv2d_last_error(None).decode())
        self.nx, self.ny = params.Nx, params.Ny

    def _check(self, rc):
        if rc != 0:
            raise Fv2dError(rc, self._lib.fv2d_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self._lib.fv2d_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_stream(self, stream_ptr):
        """Queue the context's work on a caller's CUDA stream (0: its own)."""
        self._check(self._lib.fv2d_set_stream(self.h, C.c_void_p(stream_ptr)))

    def init_problem(self, name):
        """InitFunctor::init + primToCons (Init.h:310-358) for a problem name or id."""
        pb = PROBLEMS[name] if isinstance(name, str) else int(name)
        self._check(self._lib.fv2d_init_problem(self.h, pb))

    def set_prim(self, q):
        """Replace the state by the interior primitives q (Ny, Nx, 4) = rho, u, v, p."""
        q = np.ascontiguousarray(q, dtype=np.float64)
        if q.shape != (self.ny, self.nx, 4):
            raise ValueError(f"expected shape {(self.ny, self.nx, 4)}, got {q.shape}")
        self._check(self._lib.fv2d_set_prim(self.h, _ptr(q)))

    def set_prim_ptr(self, host_ptr):
        """set_prim from a host address (page-locked memory is read by the device directly)."""
        self._check(self._lib.fv2d_set_prim(self.h, C.cast(C.c_void_p(host_ptr), _dp)))

    def prefetch_prim_ptr(self, host_ptr):
        """Start copying the next input (page-locked host address) into the
        staging buffer while queued work runs; the next set_prim_ptr with
        the same address builds the state from it."""
        self._check(self._lib.fv2d_prefetch_prim(self.h, C.c_void_p(host_ptr)))

    def get_prim_ptr(self, host_ptr):
        """get_prim into a host address (the registered host mirror is returned without a copy)."""
        self._check(self._lib.fv2d_get_prim(self.h, C.cast(C.c_void_p(host_ptr), _dp)))

    def set_host_mirror(self, host_ptr):
        """Register a page-locked (Ny, Nx, 4) float64 host array that every
        update also writes the new primitives into (0 detaches)."""
        self._check(self._lib.fv2d_set_host_mirror(self.h, C.c_void_p(host_ptr) if host_ptr else None))

    def set_prim_device(self, dev_ptr):
        """set_prim from a device array, ordered on the context's stream."""
        self._check(self._lib.fv2d_set_prim_device(self.h, C.c_void_p(dev_ptr)))

    def get_prim_device(self, dev_ptr):
        """get_prim into a device array (complete on return)."""
        self._check(self._lib.fv2d_get_prim_device(self.h, C.c_void_p(dev_ptr)))

    def get_prim(self):
        """Interior primitives (Ny, Nx, 4) = rho, u, v, p after the last update."""
        q = np.empty((self.ny, self.nx, 4))
        self._check(self._lib.fv2d_get_prim(self.h, _ptr(q)))
        return q

    def get_cons(self):
        """Interior conservative state (Ny, Nx, 4) = rho, rho u, rho v, E."""
        u = np.empty((self.ny, self.nx, 4))
        self._check(self._lib.fv2d_get_cons(self.h, _ptr(u)))
        return u

    def compute_dt(self):
        """(dt, inv_dt_hyp, inv_dt_tc, inv_dt_visc) -- ComputeDtFunctor::computeDt."""
        v = [C.c_double() for _ in range(4)]
        self._check(self._lib.fv2d_compute_dt(self.h, *[C.byref(x) for x in v]))
        return tuple(x.value for x in v)

    def update(self, dt):
        """update(Q, U, dt) + consToPrim + checkNegatives (asynchronous)."""
        self._check(self._lib.fv2d_update(self.h, float(dt)))

    def device_errors(self):
        """Error bits set by this context's kernels (1 = a bounded wait gave
        up, 2 = an index out of range in the bounds-check build)."""
        v = C.c_int()
        self._check(self._lib.fv2d_get_device_errors(self.h, C.byref(v)))
        return v.value

    def counters(self):
        """checkNegatives counts (SimInfo.h:602-645): negative densities, negative pressures and
        NaN values (each field of each interior cell counted).
        """
        c = (C.c_uint64 * 3)()
        self._check(self._lib.fv2d_get_counters(self.h, c))
        return list(c)

    def advance(self, max_steps, tend, next_save=-1.0, skip_first_save_check=False):
        """Device-driven main loop; returns (t, steps_done, status)."""
        t = C.c_double()
        n = C.c_int()
        s = C.c_int()
        rc = self._lib.fv2d_advance(self.h, int(max_steps), float(tend), float(next_save),
                                    1 if skip_first_save_check else 0, C.byref(t), C.byref(n), C.byref(s))
        if rc != 0 and s.value != RUN_NUMERIC:
            self._check(rc)
        return t.value, n.value, s.value

    def run_async(self, n):
        """Queue n device-driven iterations without synchronising."""
        self._check(self._lib.fv2d_run_async(self.h, int(n)))

    def time(self):
        """(t, iteration) of the device-driven clock."""
        t = C.c_double()
        it = C.c_int()
        self._check(self._lib.fv2d_get_time(self.h, C.byref(t), C.byref(it)))
        return t.value, it.value

    def set_time(self, t, iteration):
        """Set the device-driven clock (a restart sets the snapshot's time and iteration)."""
        self._check(self._lib.fv2d_set_time(self.h, float(t), int(iteration)))

    def step_log(self, max_records=4096):
        """Per-iteration records of the last device-driven run: columns t, dt,
        inv_dt_hyp, negative density, negative pressure, NaN counts."""
        rec = np.empty((max_records, 6))
        n = C.c_int()
        self._check(self._lib.fv2d_get_step_log(self.h, _ptr(rec), max_records, C.byref(n)))
        return rec[: n.value].copy()
