"""Test helpers: ctypes bindings of the CPU oracle (oracle/liboracle.so), of
the reference cross-check build (oracle/_ref/libfv2d_ref.so, present only
where the reference checkout was available at build time), an .ini writer
that feeds a parameter block to the reference's own reader, and seeded
random primitive states.

Only tests, __graft_entry__.smoke() and bench.py's CPU-baseline leg use the
oracle; this module is test infrastructure.
"""
import ctypes as C
import os
import subprocess
import tempfile

import numpy as np

from fv2d_gb300._abi import Params, PROBLEMS, as_float32

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_SO = os.path.join(REPO, "oracle", "liboracle.so")
REF_SO = os.path.join(REPO, "oracle", "_ref", "libfv2d_ref.so")

_dbl_p = C.POINTER(C.c_double)


def _ptr(a):
    return a.ctypes.data_as(_dbl_p)


def build_oracle():
    subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle")], check=True)


_oracle_lib = None


def oracle_lib():
    global _oracle_lib
    if _oracle_lib is None:
        if not os.path.exists(ORACLE_SO):
            build_oracle()
        lib = C.CDLL(ORACLE_SO)
        lib.fv2d_oracle_params_default.argtypes = [C.POINTER(Params)]
        lib.fv2d_oracle_create.argtypes = [C.POINTER(Params), C.POINTER(C.c_void_p)]
        lib.fv2d_oracle_destroy.argtypes = [C.c_void_p]
        lib.fv2d_oracle_init_problem.argtypes = [C.c_void_p, C.c_int]
        lib.fv2d_oracle_set_prim.argtypes = [C.c_void_p, _dbl_p]
        lib.fv2d_oracle_get_prim.argtypes = [C.c_void_p, _dbl_p]
        lib.fv2d_oracle_get_cons.argtypes = [C.c_void_p, _dbl_p]
        lib.fv2d_oracle_compute_dt.argtypes = [C.c_void_p, _dbl_p]
        lib.fv2d_oracle_update.argtypes = [C.c_void_p, C.c_double]
        lib.fv2d_oracle_get_counters.argtypes = [C.c_void_p, C.POINTER(C.c_uint64)]
        lib.fv2d_oracle_run.argtypes = [C.c_void_p, C.c_double, C.c_int, _dbl_p, C.POINTER(C.c_int), _dbl_p]
        lib.fv2d_oracle_set_threads.argtypes = [C.c_int]
        lib.fv2d_oracle_get_threads.restype = C.c_int
        lib.fv2d_oracle_uniform.restype = C.c_double
        lib.fv2d_oracle_uniform.argtypes = [C.c_int32, C.c_int64, C.c_int32]
        _oracle_lib = lib
    return _oracle_lib


def oracle_default_params(**kw):
    p = Params()
    oracle_lib().fv2d_oracle_params_default(C.byref(p))
    return p.update(**kw)


def reference_params(**kw):
    """Parameters as the reference ends up holding them after reading an .ini
    with these values: every real-valued parameter read through GetFloat is
    float-rounded, defaults included (SimInfo.h:195-200, 356-459, 536-551)."""
    p = oracle_default_params()
    for name in _GETFLOAT_FIELDS:
        setattr(p, name, as_float32(getattr(p, name)))
    for k, v in kw.items():
        if k in _GETFLOAT_FIELDS:
            v = as_float32(v)
        setattr(p, k, v)
    return p


# Real-valued fields the reference reads through Reader::GetFloat.
_GETFLOAT_FIELDS = [
    "xmin", "xmax", "ymin", "ymax", "CFL", "tend", "save_freq", "gamma0", "epsilon",
    "epsilon_reset_negative", "fslp_K", "gx", "gy", "hot_bubble_g0", "kappa", "bctc_ymin_value",
    "bctc_ymax_value", "mu", "m1", "theta1", "m2", "theta2", "h84_pert", "c91_pert", "kh_a",
    "kh_amp", "kh_P0", "kh_rho_fac", "kh_sigma", "kh_uflow", "kh_y1", "kh_y2",
    "gresho_density", "gresho_Mach",
]


class Oracle:
    """One oracle simulation (fv2d_oracle_*)."""

    def __init__(self, params):
        self.lib = oracle_lib()
        self.p = params
        self.h = C.c_void_p()
        rc = self.lib.fv2d_oracle_create(C.byref(params), C.byref(self.h))
        if rc != 0:
            raise ValueError(f"fv2d_oracle_create failed ({rc})")
        self.nx, self.ny = params.Nx, params.Ny

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.fv2d_oracle_destroy(self.h)
            self.h = None

    def init_problem(self, name):
        pb = PROBLEMS[name] if isinstance(name, str) else name
        assert self.lib.fv2d_oracle_init_problem(self.h, pb) == 0

    def set_prim(self, q):
        q = np.ascontiguousarray(q, dtype=np.float64)
        assert q.shape == (self.ny, self.nx, 4)
        assert self.lib.fv2d_oracle_set_prim(self.h, _ptr(q)) == 0

    def get_prim(self):
        q = np.empty((self.ny, self.nx, 4))
        assert self.lib.fv2d_oracle_get_prim(self.h, _ptr(q)) == 0
        return q

    def get_cons(self):
        u = np.empty((self.ny, self.nx, 4))
        assert self.lib.fv2d_oracle_get_cons(self.h, _ptr(u)) == 0
        return u

    def compute_dt(self):
        out = np.empty(4)
        assert self.lib.fv2d_oracle_compute_dt(self.h, _ptr(out)) == 0
        return out

    def update(self, dt):
        assert self.lib.fv2d_oracle_update(self.h, dt) == 0

    def counters(self):
        c = (C.c_uint64 * 3)()
        assert self.lib.fv2d_oracle_get_counters(self.h, c) == 0
        return list(c)

    def run(self, tend, max_steps, t0=0.0):
        t = C.c_double(t0)
        n = C.c_int(0)
        dts = np.empty(max(max_steps, 1))
        assert self.lib.fv2d_oracle_run(self.h, tend, max_steps, C.byref(t), C.byref(n), _ptr(dts)) == 0
        return t.value, dts[: n.value].copy()


_ref_lib = None


REF_OMP_SO = os.path.join(REPO, "oracle", "_ref", "libfv2d_ref_omp.so")
_ref_libs = {}


def ref_available(path=None):
    return os.path.exists(path or REF_SO)


def ref_lib(path=None):
    """The reference-header library: the serial parity build, or another
    build of the same sources (e.g. REF_OMP_SO, OpenMP over rows)."""
    global _ref_lib
    path = path or REF_SO
    if path != REF_SO:
        if path not in _ref_libs:
            _ref_libs[path] = _bind_ref(C.CDLL(path))
        return _ref_libs[path]
    if _ref_lib is None:
        _ref_lib = _bind_ref(C.CDLL(REF_SO))
    return _ref_lib


def _bind_ref(lib):
    lib.fv2d_ref_create.restype = C.c_void_p
    lib.fv2d_ref_create.argtypes = [C.c_char_p]
    lib.fv2d_ref_destroy.argtypes = [C.c_void_p]
    lib.fv2d_ref_dims.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    lib.fv2d_ref_param.argtypes = [C.c_void_p, C.c_char_p, _dbl_p]
    lib.fv2d_ref_init.argtypes = [C.c_void_p]
    lib.fv2d_ref_set_prim.argtypes = [C.c_void_p, _dbl_p]
    lib.fv2d_ref_get_prim.argtypes = [C.c_void_p, _dbl_p]
    lib.fv2d_ref_get_cons.argtypes = [C.c_void_p, _dbl_p]
    lib.fv2d_ref_compute_dt.restype = C.c_double
    lib.fv2d_ref_compute_dt.argtypes = [C.c_void_p, C.c_int]
    lib.fv2d_ref_update.argtypes = [C.c_void_p, C.c_double]
    return lib


_BC = {0: "absorbing", 1: "reflecting", 2: "periodic"}
_RECON = {0: "pcm", 1: "pcm_wb", 2: "plm"}
_RS = {0: "hll", 1: "hllc", 2: "fslp"}
_TS = {0: "euler", 1: "RK2"}
_GRAV = {0: "none", 1: "constant", 2: "analytical"}
_BCTC = {0: "none", 1: "fixed_temperature", 2: "fixed_gradient"}
_TCM = {0: "constant", 1: "B02"}


def params_to_ini(p, problem="blast"):
    """.ini text that makes the reference's readInifile produce parameters p
    (up to the float rounding of GetFloat)."""
    r = repr
    return f"""[mesh]
Nx={p.Nx}
Ny={p.Ny}
Nghosts={p.Nghosts}
xmin={r(p.xmin)}
xmax={r(p.xmax)}
ymin={r(p.ymin)}
ymax={r(p.ymax)}

[run]
tend={r(p.tend)}
save_freq={r(p.save_freq)}
boundaries_x={_BC[p.boundary_x]}
boundaries_y={_BC[p.boundary_y]}

[solvers]
CFL={r(p.CFL)}
reconstruction={_RECON[p.reconstruction]}
riemann_solver={_RS[p.riemann_solver]}
time_stepping={_TS[p.time_stepping]}

[physics]
gamma0={r(p.gamma0)}
problem={problem}
well_balanced_flux_at_y_bc={'true' if p.well_balanced_flux_at_y_bc else 'false'}
fslp_K={r(p.fslp_K)}

[gravity]
mode={_GRAV[p.gravity_mode]}
gx={r(p.gx)}
gy={r(p.gy)}

[hot_bubble]
g0={r(p.hot_bubble_g0)}

[thermal_conduction]
active={'true' if p.thermal_conductivity_active else 'false'}
conductivity_mode={_TCM[p.thermal_conductivity_mode]}
kappa={r(p.kappa)}
bc_ymin={_BCTC[p.bctc_ymin]}
bc_ymax={_BCTC[p.bctc_ymax]}
bc_ymin_value={r(p.bctc_ymin_value)}
bc_ymax_value={r(p.bctc_ymax_value)}

[viscosity]
active={'true' if p.viscosity_active else 'false'}
mu={r(p.mu)}

[misc]
epsilon={r(p.epsilon)}
seed={p.seed}
log_frequency={p.log_frequency}
epsilon_reset_negative={r(p.epsilon_reset_negative)}

[polytrope]
m1={r(p.m1)}
theta1={r(p.theta1)}
m2={r(p.m2)}
theta2={r(p.theta2)}

[gresho_vortex]
density={r(p.gresho_density)}
Mach={r(p.gresho_Mach)}

[kelvin_helmholtz]
a={r(p.kh_a)}
amp={r(p.kh_amp)}
P0={r(p.kh_P0)}
rho_fac={r(p.kh_rho_fac)}
sigma={r(p.kh_sigma)}

[kelvin_helmholts]
uflow={r(p.kh_uflow)}
y1={r(p.kh_y1)}
y2={r(p.kh_y2)}

[H84]
perturbation={r(p.h84_pert)}

[C91]
perturbation={r(p.c91_pert)}
"""


class RefSim:
    """The reference's own headers driven through oracle/_ref (CPU, serial)."""

    def __init__(self, params, problem="blast", lib_path=None):
        self.lib = ref_lib(lib_path)
        fd, self.path = tempfile.mkstemp(suffix=".ini")
        with os.fdopen(fd, "w") as f:
            f.write(params_to_ini(params, problem))
        self.h = self.lib.fv2d_ref_create(self.path.encode())
        if not self.h:
            raise ValueError("reference rejected the .ini")
        self.nx, self.ny = params.Nx, params.Ny

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.fv2d_ref_destroy(self.h)
            self.h = None
        if getattr(self, "path", None) and os.path.exists(self.path):
            os.unlink(self.path)

    def param(self, name):
        v = C.c_double()
        assert self.lib.fv2d_ref_param(self.h, name.encode(), C.byref(v)) == 0
        return v.value

    def init(self):
        assert self.lib.fv2d_ref_init(self.h) == 0

    def set_prim(self, q):
        q = np.ascontiguousarray(q, dtype=np.float64)
        assert self.lib.fv2d_ref_set_prim(self.h, _ptr(q)) == 0

    def get_prim(self):
        q = np.empty((self.ny, self.nx, 4))
        self.lib.fv2d_ref_get_prim(self.h, _ptr(q))
        return q

    def get_cons(self):
        u = np.empty((self.ny, self.nx, 4))
        self.lib.fv2d_ref_get_cons(self.h, _ptr(u))
        return u

    def compute_dt(self, diag=False):
        return self.lib.fv2d_ref_compute_dt(self.h, 1 if diag else 0)

    def update(self, dt):
        self.lib.fv2d_ref_update(self.h, dt)


def random_prim(ny, nx, seed, rho=(0.5, 2.0), vel=0.8, prs=(0.3, 3.0), smooth=False):
    """Seeded random valid primitive state (rho > 0, p > 0)."""
    rng = np.random.default_rng(seed)
    q = np.empty((ny, nx, 4))
    if smooth:
        y, x = np.mgrid[0:ny, 0:nx]
        ph = rng.uniform(0, 2 * np.pi, 4)
        q[..., 0] = 1.0 + 0.3 * np.sin(2 * np.pi * x / nx + ph[0]) * np.cos(2 * np.pi * y / ny + ph[1])
        q[..., 1] = 0.3 * np.sin(2 * np.pi * y / ny + ph[2])
        q[..., 2] = 0.3 * np.cos(2 * np.pi * x / nx + ph[3])
        q[..., 3] = 1.0 + 0.2 * np.cos(2 * np.pi * (x / nx + y / ny))
    else:
        q[..., 0] = rng.uniform(*rho, (ny, nx))
        q[..., 1] = rng.uniform(-vel, vel, (ny, nx))
        q[..., 2] = rng.uniform(-vel, vel, (ny, nx))
        q[..., 3] = rng.uniform(*prs, (ny, nx))
    return q


def bits_equal(a, b):
    """Bitwise equality of two float64 arrays (NaNs with equal payloads
    compare equal; +0.0 and -0.0 compare equal)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    if a.shape != b.shape:
        return False
    same = (a == b) | (np.isnan(a) & np.isnan(b))
    return bool(same.all())


def max_rel_diff(a, b, floor=1e-300):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.maximum(np.abs(b), floor)
    return float(np.max(np.abs(a - b) / den)) if a.size else 0.0
