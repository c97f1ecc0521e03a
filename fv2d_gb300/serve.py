"""ctypes binding of the batched FP32 service (include/fv2d_serve.h) and the
seeded request stream used by the benchmark and the tests."""
import ctypes as C
import math

import numpy as np

from . import lib as _lib_loader
from ._abi import ERR_STATE, Params, PROBLEMS, as_float32


class ServerConfig(C.Structure):
    _fields_ = [("struct_size", C.c_uint32), ("device", C.c_int32), ("budget_bytes", C.c_double),
                ("max_sims", C.c_int32), ("autotune", C.c_int32), ("steps_per_replay", C.c_int32),
                ("tile_config", C.c_int32), ("active_cells", C.c_double), ("single_launch", C.c_int32),
                ("band_rows", C.c_int32)]


class Request(C.Structure):
    _fields_ = [("struct_size", C.c_uint32), ("problem", C.c_int32), ("params", Params),
                ("max_steps", C.c_int32), ("lowmach", C.c_int32), ("tend", C.c_double)]


class Result(C.Structure):
    _fields_ = [("id", C.c_int64), ("status", C.c_int32), ("steps", C.c_int32), ("t", C.c_double),
                ("submit_s", C.c_double), ("admit_s", C.c_double), ("done_s", C.c_double),
                ("cons0", C.c_double * 4), ("cons1", C.c_double * 4), ("negatives", C.c_uint64),
                ("Nx", C.c_int32), ("Ny", C.c_int32), ("bucket", C.c_int32), ("lane", C.c_int32)]

    def as_dict(self):
        d = {n: getattr(self, n) for n, _ in self._fields_}
        d["cons0"] = list(self.cons0)
        d["cons1"] = list(self.cons1)
        return d


class Stats(C.Structure):
    _fields_ = [("submitted", C.c_int64), ("admitted", C.c_int64), ("completed", C.c_int64),
                ("failed", C.c_int64), ("active", C.c_int32), ("queued", C.c_int32),
                ("cell_updates", C.c_double), ("busy_s", C.c_double), ("bytes_in_use", C.c_double),
                ("bytes_reserved", C.c_double), ("bucket_cfg", C.c_int32 * 4), ("replays", C.c_int32),
                ("ext_cfg", C.c_int32), ("diff_cfg", C.c_int32 * 4)]


def _bind(L):
    if getattr(L, "_serve_bound", False):
        return L
    vp = C.c_void_p
    L.fv2d_server_create.argtypes = [C.POINTER(ServerConfig), C.POINTER(vp)]
    L.fv2d_server_destroy.argtypes = [vp]
    L.fv2d_server_submit.argtypes = [vp, C.POINTER(Request), C.POINTER(C.c_int64)]
    L.fv2d_server_poll.argtypes = [vp, C.POINTER(Result), C.c_int, C.POINTER(C.c_int)]
    L.fv2d_server_drain.argtypes = [vp, C.c_double]
    L.fv2d_server_get_prim.argtypes = [vp, C.c_int64, C.POINTER(C.c_double)]
    L.fv2d_server_release.argtypes = [vp, C.c_int64]
    L.fv2d_server_get_stats.argtypes = [vp, C.POINTER(Stats)]
    L.fv2d_server_last_error.argtypes = [vp, C.c_char_p, C.c_int]
    L.fv2d_server_check_request.argtypes = [C.POINTER(Request), C.c_char_p, C.c_int]
    L.fv2d_server_inject_fault.argtypes = [vp]
    L.fv2d_server_set_tile_wait_limit.argtypes = [vp, C.c_uint32]
    L.fv2d_server_config_name.argtypes = [C.c_int]
    L.fv2d_server_config_name.restype = C.c_char_p
    L.fv2d_server_config_families.argtypes = [C.c_int]
    L.fv2d_server_config_families.restype = C.c_int
    L._serve_bound = True
    return L


def check_request(req):
    """Why the service would refuse a Request ('' when it accepts it); needs
    no server or GPU."""
    buf = C.create_string_buffer(256)
    _bind(_lib_loader()).fv2d_server_check_request(C.byref(req), buf, len(buf))
    return buf.value.decode()


def config_name(index):
    v = _bind(_lib_loader()).fv2d_server_config_name(index)
    return v.decode() if v else None


FAMILIES = ("plain", "diffusive", "extended")


def config_families(name):
    """The kernel families (of FAMILIES) that configuration `name` serves."""
    names = config_names()
    if name not in names:
        raise ValueError(f"unknown configuration {name!r}; known: {names}")
    mask = _bind(_lib_loader()).fv2d_server_config_families(names.index(name))
    return [f for k, f in enumerate(FAMILIES) if (mask >> k) & 1]


def config_names():
    """Names of the kernel configurations, by index."""
    out = []
    while True:
        n = config_name(len(out))
        if n is None:
            return out
        out.append(n)


class Server:
    """A running batched service on one GPU."""

    def __init__(self, budget_bytes=150e9, device=0, max_sims=4096, autotune=True, steps_per_replay=0,
                 tile_config=None, active_cells=0.0, single_launch=False, band_rows=0):
        """tile_config: name of a kernel configuration (config_name) to use for
        every grid-size bucket instead of the defaults or the autotuner.
        active_cells: 0 advances every admitted request at every step; a
        positive value schedules shortest remaining work first, about that
        many cells per step.
        single_launch: every request of a kernel family in one work list and
        one persistent launch per step (instead of one per grid-size bucket).
        band_rows: rows per work item of the march kernels (0: chosen per
        lane to fill whole waves of resident warps)."""
        self.L = _bind(_lib_loader())
        forced = 0
        if tile_config is not None:
            names = config_names()
            if tile_config not in names:
                raise ValueError(f"unknown tile configuration {tile_config!r}; known: {names}")
            forced = names.index(tile_config) + 1
        cfg = ServerConfig(C.sizeof(ServerConfig), device, float(budget_bytes), max_sims, 1 if autotune else 0,
                           steps_per_replay, forced, float(active_cells), 1 if single_launch else 0, int(band_rows))
        self.h = C.c_void_p()
        rc = self.L.fv2d_server_create(C.byref(cfg), C.byref(self.h))
        if rc != 0:
            raise RuntimeError(f"fv2d_server_create failed ({rc})")
        self._n = {}

    def close(self):
        if getattr(self, "h", None):
            self.L.fv2d_server_destroy(self.h)
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

    def submit(self, problem, params, max_steps, tend=0.0, lowmach=False):
        pb = PROBLEMS[problem] if isinstance(problem, str) else int(problem)
        r = Request(C.sizeof(Request), pb, params, int(max_steps), 1 if lowmach else 0, float(tend))
        i = C.c_int64()
        rc = self.L.fv2d_server_submit(self.h, C.byref(r), C.byref(i))
        if rc == ERR_STATE:
            raise RuntimeError(f"the service has stopped: {self.last_error()}")
        if rc != 0:
            why = check_request(r)
            raise ValueError(f"request rejected ({rc}{': ' + why if why else ''})")
        self._n[i.value] = (params.Ny, params.Nx)
        return i.value

    def poll(self, max_results=1024):
        out = (Result * max_results)()
        n = C.c_int()
        self.L.fv2d_server_poll(self.h, out, max_results, C.byref(n))
        return [out[k] for k in range(n.value)]

    def drain(self, timeout_s=600.0):
        """0 once nothing is queued or running; ERR_STATE on timeout; the
        stopping code (ERR_CUDA, ERR_NOMEM) once the service has stopped."""
        return self.L.fv2d_server_drain(self.h, float(timeout_s))

    def last_error(self):
        """Why the service stopped ('' while it runs)."""
        buf = C.create_string_buffer(512)
        self.L.fv2d_server_last_error(self.h, buf, len(buf))
        return buf.value.decode(errors="replace")

    def inject_fault(self):
        """Test hook: the worker stops as if a CUDA call had failed."""
        self.L.fv2d_server_inject_fault(self.h)

    def set_tile_wait_limit(self, polls):
        """Test hook: polls of a TMA tile copy's barrier before the request
        it belongs to is failed (default 2^24; 0 = none)."""
        self.L.fv2d_server_set_tile_wait_limit(self.h, int(polls))

    def get_prim(self, rid):
        ny, nx = self._n[rid]
        q = np.empty((ny, nx, 4))
        rc = self.L.fv2d_server_get_prim(self.h, rid, q.ctypes.data_as(C.POINTER(C.c_double)))
        if rc != 0:
            raise KeyError(rid)
        return q

    def release(self, rid):
        self.L.fv2d_server_release(self.h, rid)

    def stats(self):
        s = Stats()
        self.L.fv2d_server_get_stats(self.h, C.byref(s))
        return s


def stream_requests(n=512, rate=200.0, seed=12345, nmin=64, nmax=1024, steps=(200, 2000)):
    """The benchmark's request stream: a seeded Poisson arrival process;
    grid N log-uniform in [nmin, nmax] rounded to a multiple of 32; initial
    condition uniform over Sod (density ratio 2..20), Sedov (E0 0.5..2),
    Kelvin-Helmholtz (shear speed 0.2..1) and Gresho (rho = 1, Mach
    0.01..0.1); gamma uniform in [1.3, 1.67]; 200..2000 steps.  Returns a
    list of dicts with arrival time, problem, params and step count."""
    from . import default_params, PLM, HLLC, BC_ABSORBING, BC_REFLECTING, BC_PERIODIC
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for k in range(n):
        t += rng.exponential(1.0 / rate)
        N = int(round(math.exp(rng.uniform(math.log(nmin), math.log(nmax))) / 32.0)) * 32
        N = min(max(N, nmin), nmax)
        kind = ["sod", "sedov", "kh", "gresho"][int(rng.integers(0, 4))]
        gamma = float(rng.uniform(1.3, 1.67))
        nsteps = int(rng.integers(steps[0], steps[1] + 1))
        f = as_float32
        p = default_params(Nx=N, Ny=N, gamma0=f(gamma), CFL=f(0.8), reconstruction=PLM, riemann_solver=HLLC)
        lowmach = False
        if kind == "sod":
            ratio = float(rng.uniform(2.0, 20.0))
            p.update(boundary_x=BC_ABSORBING, boundary_y=BC_PERIODIC, sod_rho_left=1.0, sod_p_left=1.0,
                     sod_rho_right=1.0 / ratio, sod_p_right=0.1)
            problem = "sod_x"
        elif kind == "sedov":
            p.update(boundary_x=BC_REFLECTING, boundary_y=BC_REFLECTING, sedov_E0=float(rng.uniform(0.5, 2.0)))
            problem = "sedov"
        elif kind == "kh":
            p.update(boundary_x=BC_PERIODIC, boundary_y=BC_PERIODIC, khs_u=float(rng.uniform(0.2, 1.0)),
                     seed=int(rng.integers(1, 1 << 30)))
            problem = "kh_step"
        else:
            p.update(boundary_x=BC_PERIODIC, boundary_y=BC_PERIODIC, gresho_density=1.0,
                     gresho_Mach=f(float(rng.uniform(0.01, 0.1))))
            problem = "gresho_vortex"
            lowmach = True
        out.append(dict(arrival=t, problem=problem, params=p, steps=nsteps, N=N, kind=kind, lowmach=lowmach))
    return out
