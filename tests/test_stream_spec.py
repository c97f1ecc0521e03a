"""The served benchmark's request stream (fv2d_gb300.serve.stream_requests)
against its stated specification, without a GPU: 512 requests arriving as a
seeded Poisson process at 200/s; N log-uniform in [64, 1024], a multiple of
32; initial conditions uniform over Sod (density ratio 2..20), Sedov
(E0 0.5..2), Kelvin-Helmholtz (shear speed 0.2..1) and Gresho (rho = 1,
Mach 0.01..0.1); gamma in [1.3, 1.67]; 200..2000 steps."""
import math

import numpy as np

from fv2d_gb300 import BC_ABSORBING, BC_PERIODIC, BC_REFLECTING, HLLC, PLM
from fv2d_gb300.serve import stream_requests


def test_stream_follows_its_specification():
    reqs = stream_requests()
    assert len(reqs) == 512
    t = np.array([r["arrival"] for r in reqs])
    gaps = np.diff(np.concatenate([[0.0], t]))
    assert np.all(gaps > 0)
    assert abs(np.mean(gaps) - 1 / 200.0) < 0.15 / 200.0          # mean inter-arrival 5 ms
    assert abs(np.std(gaps) / np.mean(gaps) - 1.0) < 0.15           # exponential: coefficient of variation 1
    Ns = np.array([r["N"] for r in reqs])
    assert np.all(Ns % 32 == 0) and Ns.min() >= 64 and Ns.max() <= 1024
    logs = np.log(Ns)
    assert abs(np.median(logs) - 0.5 * (math.log(64) + math.log(1024))) < 0.25   # log-uniform: median near 256
    kinds = [r["kind"] for r in reqs]
    for k in ("sod", "sedov", "kh", "gresho"):
        assert 0.18 < kinds.count(k) / len(reqs) < 0.32, k
    for r in reqs:
        p = r["params"]
        assert p.Nx == p.Ny == r["N"] and p.reconstruction == PLM and p.riemann_solver == HLLC
        assert 1.3 <= p.gamma0 <= 1.67 and 200 <= r["steps"] <= 2000
        if r["kind"] == "sod":
            assert r["problem"] == "sod_x" and (p.boundary_x, p.boundary_y) == (BC_ABSORBING, BC_PERIODIC)
            assert 2.0 <= p.sod_rho_left / p.sod_rho_right <= 20.0 + 1e-9
        elif r["kind"] == "sedov":
            assert r["problem"] == "sedov" and (p.boundary_x, p.boundary_y) == (BC_REFLECTING, BC_REFLECTING)
            assert 0.5 <= p.sedov_E0 <= 2.0
        elif r["kind"] == "kh":
            assert r["problem"] == "kh_step" and 0.2 <= p.khs_u <= 1.0
        else:
            assert r["problem"] == "gresho_vortex" and p.gresho_density == 1.0 and r["lowmach"]
            assert 0.0099 <= p.gresho_Mach <= 0.1001
    # seeded: the same stream every time
    again = stream_requests()
    assert [(a["arrival"], a["N"], a["steps"]) for a in again] == [(b["arrival"], b["N"], b["steps"]) for b in reqs]
