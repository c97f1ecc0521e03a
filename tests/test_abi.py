"""C-ABI checks that need no GPU: the library builds and loads, exports every
entry point declared in include/*.h, and agrees with the Python mirror of the
parameter block."""
import ctypes as C
import glob
import os
import re
import subprocess

import pytest

from fv2d_testlib import REPO, reference_params
from fv2d_gb300 import _abi


@pytest.fixture(scope="module")
def libs():
    from fv2d_gb300 import build as b
    b.build()
    import fv2d_gb300
    return fv2d_gb300.lib()


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(REPO, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w \*]*?\b(fv2d_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_exports_every_declared_symbol(libs):
    names = declared_functions()
    assert "fv2d_create" in names and "fv2d_update" in names and "fv2d_compute_dt" in names
    from fv2d_gb300 import LIB_PATH
    out = subprocess.run(["nm", "-D", "--defined-only", LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (fv2d_\w+)", out))
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    for n in names:
        assert hasattr(libs, n)


def test_params_layout_matches_header(libs):
    assert libs.fv2d_params_size() == C.sizeof(_abi.Params)
    text = open(os.path.join(REPO, "include", "fv2d_types.h")).read()
    body = text[text.index("typedef struct fv2d_params {"):text.index("} fv2d_params;")]
    fields = []
    for line in body.splitlines()[1:]:
        line = re.sub(r"/\*.*?\*/", "", line).strip()
        m = re.match(r"(uint32_t|int32_t|double)\s+(.*);", line)
        if m:
            fields += [(n.strip(), m.group(1)) for n in m.group(2).split(",")]
    ctypes_of = {"uint32_t": C.c_uint32, "int32_t": C.c_int32, "double": C.c_double}
    assert [(n, ctypes_of[t]) for n, t in fields] == list(_abi.Params._fields_)


def test_defaults_are_the_references_effective_values(libs):
    from fv2d_gb300 import default_params
    p = default_params()
    r = reference_params()
    for name, _ in _abi.Params._fields_:
        assert getattr(p, name) == getattr(r, name), name
    assert p.gamma0 == float(C.c_float(5.0 / 3.0).value)
    assert p.CFL == float(C.c_float(0.8).value)


def test_build_info(libs):
    from fv2d_gb300 import build_info
    s = build_info()
    assert "sm_103a" in s and "TMA" in s


def test_create_rejects_bad_params_without_gpu(libs):
    """Validation happens before any CUDA call."""
    from fv2d_gb300 import Fv2dError, Simulation, default_params
    for bad in (dict(Nx=1), dict(Nghosts=1), dict(riemann_solver=7), dict(boundary_x=5), dict(xmax=-1.0)):
        with pytest.raises(Fv2dError) as e:
            Simulation(default_params(**bad))
        assert e.value.code == _abi.ERR_INVALID


def _header_fields(header, struct):
    text = open(os.path.join(REPO, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    body = text[text.index(f"typedef struct {struct} {{"):text.index(f"}} {struct};")]
    fields = []
    for line in body.splitlines()[1:]:
        m = re.match(r"\s*(uint32_t|int32_t|double)\s+(.*);", line)
        if m:
            fields += [(n.strip(), m.group(1)) for n in m.group(2).split(",")]
    return fields


def test_server_config_layout_matches_header(libs):
    from fv2d_gb300.serve import ServerConfig
    ctypes_of = {"uint32_t": C.c_uint32, "int32_t": C.c_int32, "double": C.c_double}
    fields = _header_fields("fv2d_serve.h", "fv2d_server_config")
    assert [(n, ctypes_of[t]) for n, t in fields] == list(ServerConfig._fields_)


def test_server_rejects_bad_configs_without_gpu(libs):
    """Checked before any CUDA call: size, table capacity, budget, scheduling cap, launch form, band height."""
    from fv2d_gb300.serve import ServerConfig, _bind
    lib = _bind(libs)
    good = dict(device=0, budget_bytes=1e9, max_sims=16, autotune=0, steps_per_replay=0, tile_config=0,
                active_cells=0.0)
    for bad in (dict(max_sims=0), dict(max_sims=1 << 20), dict(budget_bytes=0.0), dict(active_cells=-1.0),
                dict(active_cells=float("nan")), dict(active_cells=float("inf")), dict(single_launch=2),
                dict(band_rows=-1), dict(band_rows=4), dict(band_rows=65)):
        kw = dict(good, **bad)
        cfg = ServerConfig(C.sizeof(ServerConfig), **kw)
        h = C.c_void_p()
        assert lib.fv2d_server_create(C.byref(cfg), C.byref(h)) == _abi.ERR_INVALID, bad
    cfg = ServerConfig(C.sizeof(ServerConfig) - 8, **good)
    h = C.c_void_p()
    assert lib.fv2d_server_create(C.byref(cfg), C.byref(h)) == _abi.ERR_INVALID
    # calls on no server
    buf = C.create_string_buffer(16)
    assert lib.fv2d_server_last_error(None, buf, 16) == _abi.ERR_INVALID
    assert lib.fv2d_server_inject_fault(None) == _abi.ERR_INVALID
    assert lib.fv2d_server_drain(None, 1.0) == _abi.ERR_INVALID


def test_no_cpu_fallback_without_a_gpu(libs):
    """Without a usable GPU the library refuses loudly (FV2D_ERR_CUDA and the
    CUDA message); nothing falls back to a CPU path."""
    from fv2d_gb300 import Fv2dError, Simulation, default_params
    try:
        s = Simulation(default_params(Nx=32, Ny=32))
    except Fv2dError as e:
        assert e.code == _abi.ERR_CUDA and "CUDA" in str(e)
        return
    s.close()
    pytest.skip("a GPU is present")


def test_server_has_no_cpu_fallback_without_a_gpu(libs):
    """A valid server configuration without a usable GPU: FV2D_ERR_CUDA, no
    server, no worker thread."""
    from fv2d_gb300.serve import ServerConfig, _bind
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = _bind(libs)
    cfg = ServerConfig(C.sizeof(ServerConfig), 0, 1e9, 16, 0, 0, 0, 0.0)
    h = C.c_void_p()
    assert lib.fv2d_server_create(C.byref(cfg), C.byref(h)) == _abi.ERR_CUDA
    assert not h.value


def test_server_request_checks_without_a_server(libs):
    """fv2d_server_check_request: the request checks of fv2d_server_submit,
    with their reasons, callable without a server or a GPU."""
    import fv2d_gb300 as fv
    from fv2d_gb300.serve import Request, check_request, _bind
    lib = _bind(libs)

    def req(**kw):
        base = dict(Nx=128, Ny=128, reconstruction=fv.PLM, riemann_solver=fv.HLLC)
        base.update(kw)
        return Request(C.sizeof(Request), fv.PROBLEMS["sedov"], fv.default_params(**base), 10, 0, 0.0)

    assert check_request(req()) == ""
    buf = C.create_string_buffer(64)
    assert lib.fv2d_server_check_request(C.byref(req()), buf, 64) == _abi.OK
    # every scheme, physics switch and rectangular grid is accepted
    for kw in (dict(riemann_solver=fv.FSLP), dict(Nx=100, Ny=36), dict(Ny=96), dict(time_stepping=fv.TS_RK2),
               dict(reconstruction=fv.MUSCL_HANCOCK), dict(gravity_mode=fv.GRAV_ANALYTICAL),
               dict(well_balanced_flux_at_y_bc=1), dict(thermal_conductivity_active=1, kappa=1e-3,
                                                        thermal_conductivity_mode=fv.TCM_B02,
                                                        bctc_ymin=fv.BCTC_FIXED_TEMPERATURE)):
        assert check_request(req(**kw)) == "", kw
    cases = [(dict(Nx=8), "[16, 8192]"), (dict(Ny=8193), "[16, 8192]"), (dict(reconstruction=9), "reconstruction"),
             (dict(riemann_solver=3), "riemann_solver")]
    for kw, why in cases:
        r = req(**kw)
        assert lib.fv2d_server_check_request(C.byref(r), buf, 64) == _abi.ERR_UNSUPPORTED, kw
        assert why in buf.value.decode() and why in check_request(r), (kw, buf.value)
    bad = req()
    bad.struct_size -= 8
    assert "struct_size" in check_request(bad)
    neg = req()
    neg.max_steps = -1
    assert "max_steps" in check_request(neg)
    assert lib.fv2d_server_check_request(None, buf, 64) == _abi.ERR_INVALID
    assert lib.fv2d_server_check_request(C.byref(req()), None, 0) == _abi.OK
    assert lib.fv2d_server_check_request(C.byref(req()), buf, -1) == _abi.ERR_INVALID


def test_kernel_configurations_without_gpu(libs):
    """The service's kernel configurations: unique names, every kernel
    family served by at least one, the march kernels named by strip,
    threads per CTA and CTAs per SM, and a plain-only two-column one."""
    from fv2d_gb300.serve import config_names, config_families, FAMILIES, _bind
    names = config_names()
    assert len(names) == len(set(names)) and len(names) >= 3
    fams = {n: config_families(n) for n in names}
    for f in FAMILIES:
        assert any(f in v for v in fams.values()), f
    assert all(fams[n] for n in names)
    assert fams["60/32x16/march2"] == ["plain"]
    assert fams["60/32x10/march2-diff"] == ["diffusive"]
    assert fams["28/32x20/march"] == ["plain", "diffusive"]
    assert fams["28/64x8/march-ext"] == ["extended"]
    lib = _bind(libs)
    assert lib.fv2d_server_config_families(-1) == -1
    assert lib.fv2d_server_config_families(len(names)) == -1
