"""The fv2d_gpu driver end to end (main.cpp's role): .ini in, HDF5 snapshots
and the reference's console lines out, restart from a snapshot.  Every
snapshot is compared bit for bit with the oracle run through the same loop
(main.cpp:62-84) and the same restart sequence (IOManager.h:284-398)."""
import os
import subprocess

import pytest

from fv2d_testlib import Oracle, bits_equal, reference_params
from test_io import io_lib, read

pytestmark = pytest.mark.gpu

INI = """[mesh]
Nx=64
Ny=8
xmin=0.0
xmax=1.0
ymin=0.0
ymax=0.125

[run]
tend=0.05
save_freq=0.01
boundaries_x=absorbing
boundaries_y=periodic
output_path={out}
output_filename={name}
{restart}

[solvers]
riemann_solver=hllc
reconstruction=plm
CFL=0.8

[physics]
gamma0=1.4
problem=sod_x

[misc]
log_frequency=3
"""


def oracle_loop(o, p, t, ite, next_save):
    """main.cpp:62-84 on the oracle; returns snapshots {ite: (t, q)}, dt log
    lines, final t, next ite."""
    snaps, lines, next_log = {}, [], 0
    while t + p.epsilon < p.tend:
        save_needed = t + p.epsilon > next_save
        d = o.compute_dt()
        if next_log == 0:
            lines.append("Computing dts at (t=%g) : dt_hyp=%g" % (t, 1.0 / d[1]))
        next_log = p.log_frequency if next_log == 0 else next_log - 1
        if save_needed:
            snaps[ite] = (t, o.get_prim())
            ite += 1
            next_save += p.save_freq
        o.update(d[0])
        t += d[0]
    snaps[ite] = (t, o.get_prim())
    return snaps, lines, t


def run_driver(tmp_path, name, restart="", extra=()):
    from fv2d_gb300 import build as b
    b.build()
    exe = os.path.join(os.path.dirname(b.LIB), "..", "bin", "fv2d_gpu")
    ini = tmp_path / (name + ".ini.in")
    ini.write_text(INI.format(out=str(tmp_path), name=name, restart=restart))
    r = subprocess.run([exe, str(ini), *extra], cwd=str(tmp_path), capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


def test_driver_snapshots_and_log_match_oracle(gpu_lib, tmp_path):
    out = run_driver(tmp_path, "run")
    p = reference_params(Nx=64, Ny=8, ymax=0.125, tend=0.05, save_freq=0.01, boundary_x=0, boundary_y=2,
                         riemann_solver=1, reconstruction=2, CFL=0.8, gamma0=1.4, log_frequency=3)
    o = Oracle(p)
    o.init_problem("sod_x")
    snaps, lines, t_end = oracle_loop(o, p, 0.0, 0, 0.0)
    L = io_lib()
    f = str(tmp_path / "run.h5")
    for k, (t, q) in snaps.items():
        rc, qg, tg, itg, err = read(L, f + ":/ite_%04d" % k, 64, 8)
        assert rc == 0, err
        assert tg == t and itg == k
        assert bits_equal(qg, q), k
    got = [ln for ln in out.splitlines() if ln.startswith("Computing dts")]
    assert got == lines
    assert out.count(" - Saving at time ") == len(snaps) - 1
    assert ("Time at end is %g" % t_end) in out
    assert (tmp_path / "last.ini").read_text().startswith("; Parameters used for the problem: sod_x")


def test_driver_restart_matches_oracle(gpu_lib, tmp_path):
    run_driver(tmp_path, "run")
    out = run_driver(tmp_path, "run2", restart="restart_file=%s:/ite_0002" % (tmp_path / "run.h5"))
    assert "Restart at iteration 2 and time" in out
    p = reference_params(Nx=64, Ny=8, ymax=0.125, tend=0.05, save_freq=0.01, boundary_x=0, boundary_y=2,
                         riemann_solver=1, reconstruction=2, CFL=0.8, gamma0=1.4, log_frequency=3)
    L = io_lib()
    rc, q2, t2, it2, _ = read(L, str(tmp_path / "run.h5") + ":/ite_0002", 64, 8)
    assert rc == 0
    o = Oracle(p)
    o.set_prim(q2)  # restart: primitives -> boundaries -> primToCons
    snaps, _, _ = oracle_loop(o, p, t2, it2 + 1, t2 + p.save_freq)
    f = str(tmp_path / "run2.h5")
    rc, q, t, it, err = read(L, f + ":/ite_0002", 64, 8)  # the restart state, written first
    assert rc == 0 and it == 2 and t == t2 and bits_equal(q, q2), err
    for k, (t, q) in snaps.items():
        rc, qg, tg, itg, err = read(L, f + ":/ite_%04d" % k, 64, 8)
        assert rc == 0, err
        assert tg == t and itg == k and bits_equal(qg, q), k


def test_driver_metrics_log_is_the_iteration_log(gpu_lib, tmp_path):
    """--metrics FILE: one JSON line per iteration (t, dt, inverse dt,
    checkNegatives counts) equal to the oracle loop's, plus batch timings."""
    import json
    metrics = tmp_path / "m.jsonl"
    run_driver(tmp_path, "run", extra=("--metrics", str(metrics)))
    recs = [json.loads(line) for line in metrics.read_text().splitlines()]
    steps = [r for r in recs if "step" in r]
    batches = [r for r in recs if "batch_steps" in r]
    p = reference_params(Nx=64, Ny=8, ymax=0.125, tend=0.05, save_freq=0.01, boundary_x=0, boundary_y=2,
                         riemann_solver=1, reconstruction=2, CFL=0.8, gamma0=1.4, log_frequency=3)
    o = Oracle(p)
    o.init_problem("sod_x")
    t = 0.0
    ts, dts = [], []
    while t + p.epsilon < p.tend:
        d = o.compute_dt()
        ts.append(t)
        dts.append(d[0])
        o.update(d[0])
        t += d[0]
    assert [r["step"] for r in steps] == list(range(len(dts)))
    assert [r["t"] for r in steps] == ts and [r["dt"] for r in steps] == dts
    assert all(r["neg_rho"] == 0 and r["neg_p"] == 0 and r["nan"] == 0 for r in steps)
    assert sum(b["batch_steps"] for b in batches) == len(dts) and all(b["wall_s"] >= 0 for b in batches)
