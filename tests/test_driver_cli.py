"""The fv2d_gpu executable's checks that come before any GPU work, run here
without a GPU: no argument, a missing .ini, an unknown problem (the
reference's message, Init.h:303-304), an output directory that cannot be
created, and, with no usable GPU, a failure with the CUDA message after the
.ini echo (no CPU fallback)."""
import os
import subprocess

import pytest

INI = """[mesh]
Nx=32
Ny=8
[run]
tend=0.01
save_freq=0.01
boundaries_x=absorbing
boundaries_y=periodic
output_path={out}
output_filename=run
[solvers]
riemann_solver=hllc
reconstruction=plm
[physics]
gamma0=1.4
problem={problem}
"""


@pytest.fixture(scope="module")
def exe():
    from fv2d_gb300 import build as b
    b.build()
    return b.DRIVER


def run(exe, tmp_path, *args):
    return subprocess.run([exe, *map(str, args)], cwd=str(tmp_path), capture_output=True, text=True, timeout=120)


def write_ini(tmp_path, out, problem="sod_x"):
    ini = tmp_path / "case.ini"
    ini.write_text(INI.format(out=out, problem=problem))
    return ini


def test_usage_without_arguments(exe, tmp_path):
    r = run(exe, tmp_path)
    assert r.returncode == 1 and "usage: fv2d_gpu" in r.stderr


def test_missing_ini(exe, tmp_path):
    r = run(exe, tmp_path, tmp_path / "absent.ini")
    assert r.returncode == 1 and "cannot open" in r.stderr


def test_unknown_problem(exe, tmp_path):
    r = run(exe, tmp_path, write_ini(tmp_path, tmp_path / "out", problem="blastx"))
    assert r.returncode == 1 and "Error unknown problem blastx" in r.stderr
    assert not (tmp_path / "last.ini").exists()  # stopped before the echo, as the reference


def test_output_directory_that_cannot_be_created(exe, tmp_path):
    (tmp_path / "plain_file").write_text("x")
    r = run(exe, tmp_path, write_ini(tmp_path, tmp_path / "plain_file" / "out"))
    assert r.returncode == 1 and "cannot create" in r.stderr


def test_no_gpu_fails_with_the_cuda_message(exe, tmp_path):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    r = run(exe, tmp_path, write_ini(tmp_path, tmp_path / "out"))
    assert r.returncode == 1 and "CUDA" in r.stderr, r.stdout + r.stderr
    assert (tmp_path / "last.ini").exists() and (tmp_path / "out" / "run.ini").exists()
    assert not (tmp_path / "out" / "run.h5").exists()
