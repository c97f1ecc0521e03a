"""The service's HBM state arena (fv2d_gb300/csrc/arena.hpp), on the host.

The same template the service instantiates with cudaMalloc/cudaFree is
compiled here against a backend that hands out address ranges with no memory
behind them, and driven through randomised admissions and retirements of
service-sized states (grids 64..4096) under a 6.5 GB budget, with the backend
refusing now and then.  tests/arena_harness.cpp checks after every operation
that blocks never overlap, the accounting and the budget hold, the free lists
tile the chunks and stay merged, and that a refusal had a reason; at the end
every chunk is one free block again.
"""
import os
import shutil
import subprocess

import pytest

from fv2d_testlib import REPO


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    cxx = shutil.which(os.environ.get("CXX", "g++")) or shutil.which("g++")
    if not cxx:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path_factory.mktemp("arena") / "arena_harness")
    subprocess.run([cxx, "-std=c++17", "-O2", "-Wall", "-Werror", "-o", exe,
                    os.path.join(REPO, "tests", "arena_harness.cpp")], check=True)
    return exe


@pytest.mark.parametrize("seed", [1, 2, 3, 4])
def test_arena_invariants_under_random_admission_and_retirement(harness, seed):
    r = subprocess.run([harness, str(seed), "20000"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("ok ")
