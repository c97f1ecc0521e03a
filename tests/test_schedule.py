"""The service's scheduling choice (fv2d_gb300/csrc/schedule.hpp), on the
host: which resident requests advance when `active_cells` caps the cells per
step.  Checked against this restatement of the policy on random cases with
ties, caps of zero, below one request and above all of them, and no requests:
take requests by least remaining work (then lowest slot) while the cells
taken are below the cap; with no cap take every request."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from fv2d_testlib import REPO


def policy(cands, cap):
    if cap <= 0:
        return sorted(s for s, _, _ in cands)
    run, cells = [], 0.0
    for s, rem, c in sorted(cands, key=lambda x: (x[1], x[0])):
        if run and cells >= cap:
            break
        run.append(s)
        cells += c
    return sorted(run)


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    cxx = shutil.which(os.environ.get("CXX", "g++")) or shutil.which("g++")
    if not cxx:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path_factory.mktemp("schedule") / "schedule_harness")
    subprocess.run([cxx, "-std=c++17", "-O2", "-Wall", "-Werror", "-o", exe,
                    os.path.join(REPO, "tests", "schedule_harness.cpp")], check=True)
    return exe


def test_shortest_remaining_work_first_matches_the_policy(harness):
    rng = np.random.default_rng(5)
    cases = [([], 1e6), ([(3, 10.0, 4096.0)], 0.0), ([(3, 10.0, 4096.0)], 1.0)]
    for _ in range(400):
        n = int(rng.integers(1, 40))
        slots = rng.choice(4096, size=n, replace=False)
        Ns = rng.choice(np.arange(64, 1025, 32), size=n)
        steps = rng.integers(1, 5, size=n) * 100  # few distinct values: ties in remaining work
        cands = [(int(s), float(k * N * N), float(N * N)) for s, N, k in zip(slots, Ns, steps)]
        total = sum(c for _, _, c in cands)
        cap = float(rng.choice([0.0, 1.0, 0.3 * total, 0.7 * total, 2.0 * total]))
        cases.append((cands, cap))
    text = "".join(f"{len(c)} {cap!r}\n" + "".join(f"{s} {r!r} {x!r}\n" for s, r, x in c) for c, cap in cases)
    r = subprocess.run([harness], input=text, capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.split("\n")[:len(cases)]
    for (cands, cap), line in zip(cases, lines):
        got = [int(x) for x in line.split()]
        assert got == policy(cands, cap), (cands, cap)
        if cands and cap > 0:
            chosen = sum(c for s, _, c in cands if s in got)
            assert got and (chosen >= cap or len(got) == len(cands))


def band_rule(grids, warps):
    """The march lanes' band height: the tallest of 32, 24, 16, 12, 8 rows
    that gives the launch at least 2 work items per resident warp, else 8."""
    for H in (32, 24, 16, 12, 8):
        if sum(s * -(-ny // H) for s, ny in grids) >= 2.0 * warps:
            return H
    return 8


def test_band_height_matches_the_rule(harness):
    rng = np.random.default_rng(11)
    # single grids the benchmark runs: RT 1024 x 3072 on the one-column march
    # (37 strips of 28, 3040 resident warps) takes 16 rows; KH 4096^2 on the
    # two-column one (69 strips of 60, 2432 warps) 32 rows; a lone 64^2 grid 8
    cases = [([(37, 3072)], 3040.0), ([(69, 4096)], 2432.0), ([(3, 64)], 3040.0), ([(13, 768)] * 12, 2432.0)]
    expect = [16, 32, 8, 24]
    for _ in range(300):
        n = int(rng.integers(1, 60))
        strip = int(rng.choice([28, 60]))
        Ns = rng.integers(16, 2049, size=n)
        grids = [(-(-int(rng.integers(16, 2049)) // strip), int(N)) for N in Ns]
        cases.append((grids, float(rng.choice([2432.0, 3040.0, 1216.0]))))
    text = "".join(f"{len(g)} {w!r}\n" + "".join(f"{s} {ny}\n" for s, ny in g) for g, w in cases)
    r = subprocess.run([harness, "band"], input=text, capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    got = [int(x) for x in r.stdout.split()]
    assert len(got) == len(cases)
    assert got[:len(expect)] == expect
    for (grids, warps), h in zip(cases, got):
        assert h == band_rule(grids, warps), (grids, warps)
