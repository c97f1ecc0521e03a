"""The bounds-check build (-DFV2D_BOUNDS_CHECK; compute-sanitizer is not used
here): every shared-memory index and global plane index of the FP64 step is
checked on the device, a bad one recorded in the context's error bits and
skipped.  On odd grid sizes that cut tiles (down to two cells along an axis) and on every kind of step
(PCM / PLM / MUSCL-Hancock, HLL / HLLC / FSLP, Euler / RK2, gravity,
conduction, viscosity, the well-balanced boundary flux, every boundary type)
it must report nothing and produce the same bits as the normal build."""
import os
import subprocess
import sys

import numpy as np
import pytest

import golden.make_golden as G
from fv2d_testlib import bits_equal, random_prim, reference_params

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
SHAPES = [(5, 3), (17, 33), (40, 65), (2, 2), (2, 9), (9, 2)]


def cases():
    out = []
    combos = G.combo_list()[::9] + [  # MUSCL-Hancock (reconstruction 3), Euler and RK2
        dict(reconstruction=3, riemann_solver=1, time_stepping=0, boundary_x=1, boundary_y=2),
        dict(reconstruction=3, riemann_solver=0, time_stepping=1, boundary_x=2, boundary_y=0, viscosity_active=1,
             mu=1e-2)]
    for k, c in enumerate(combos):
        ny, nx = SHAPES[k % len(SHAPES)]
        out.append((c, ny, nx))
    return out


def run(q0s, lib_path=None):
    """3 steps of every case; with lib_path, through that library."""
    import fv2d_gb300 as fv
    if lib_path:
        fv.LIB_PATH = lib_path
    res, errs = [], []
    for (c, ny, nx), q0 in zip(cases(), q0s):
        p = reference_params(Nx=nx, Ny=ny, gamma0=1.4, CFL=0.6, **c)
        s = fv.Simulation(p)
        s.set_prim(q0)
        for _ in range(3):
            s.update(s.compute_dt()[0])
        res.append(s.get_prim())
        errs.append(s.device_errors())
        s.close()
    return res, errs


def test_bounds_checked_build_reports_nothing_and_matches(gpu_lib, tmp_path):
    from fv2d_gb300 import build as b
    checked = b.build(bounds_check=True)
    q0s = [random_prim(ny, nx, 31 + k) for k, (_, ny, nx) in enumerate(cases())]
    np.savez(tmp_path / "in.npz", *q0s)
    script = f"""
import sys, numpy as np
sys.path[:0] = [{os.path.dirname(HERE)!r}, {HERE!r}]
from test_bounds_check import run
d = np.load({str(tmp_path / "in.npz")!r})
res, errs = run([d["arr_%d" % k] for k in range(len(d.files))], {checked!r})
np.savez({str(tmp_path / "out.npz")!r}, errs=np.array(errs), *res)
"""
    r = subprocess.run([sys.executable, "-c", script], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    out = np.load(tmp_path / "out.npz")
    assert not out["errs"].any(), out["errs"]
    ref, errs = run(q0s)
    assert not any(errs)
    for k, q in enumerate(ref):
        assert bits_equal(out["arr_%d" % k], q), cases()[k]
