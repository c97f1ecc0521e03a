"""The allocation-free dt entry point, fv2d_compute_dt_noalloc.

It serves callers that cannot call cudaMalloc: code whose device memory is
owned by another allocator (a framework pool that accounts for every byte, a
process that reserved all device memory up front) and loops that cannot
afford the synchronisation an allocation may cause.  The caller passes a
device array of primitives and a device array for the result; the function
keeps its reduction scratch in a fixed array inside the library.

Checked here through the C-ABI against the existing entry point
(fv2d_compute_dt on a context holding the same state), bit for bit, on two
calls in a row with different states, plus the size limit.  This file is
collected last on purpose.
"""
import numpy as np
import pytest

from fv2d_testlib import Oracle, bits_equal, random_prim, reference_params

pytestmark = pytest.mark.gpu


def test_noalloc_dt_matches_compute_dt_twice(gpu_lib):
    import torch
    import fv2d_gb300 as fv

    out = torch.full((4,), -7.0, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()

    # call 1: Sedov initial state, 512 x 384, PLM/HLLC
    p1 = reference_params(Nx=512, Ny=384, gamma0=1.4, CFL=0.8, reconstruction=2, riemann_solver=1)
    s1 = fv.Simulation(p1)
    s1.init_problem("sedov")
    q1 = torch.from_numpy(s1.get_prim()).to("cuda")
    expect1 = np.array(s1.compute_dt())
    assert fv.compute_dt_noalloc(p1, q1.data_ptr(), out.data_ptr(), stream.cuda_stream) == 0
    stream.synchronize()
    assert bits_equal(out.cpu().numpy(), expect1)

    # call 2: a different state (random, after 3 updates) with conduction and
    # viscosity limits, non-power-of-two spacing
    p2 = reference_params(Nx=300, Ny=200, xmax=0.7, gamma0=1.4, CFL=0.6, thermal_conductivity_active=1,
                          kappa=1e-3, viscosity_active=1, mu=2e-3, boundary_x=2, boundary_y=0)
    s2 = fv.Simulation(p2)
    s2.set_prim(random_prim(200, 300, 21))
    for _ in range(3):
        s2.update(s2.compute_dt()[0])
    q2 = torch.from_numpy(s2.get_prim()).to("cuda")
    expect2 = np.array(s2.compute_dt())
    assert fv.compute_dt_noalloc(p2, q2.data_ptr(), out.data_ptr(), stream.cuda_stream) == 0
    stream.synchronize()
    assert bits_equal(out.cpu().numpy(), expect2)
    assert not bits_equal(expect1, expect2)


def test_noalloc_dt_skips_a_nan_cell_like_compute_dt(gpu_lib):
    """A state with one NaN cell: the reference's max reduction (fmax,
    ComputeDt.h:46-48) skips it, and so do both entry points -- same bits,
    also against the oracle."""
    import torch
    import fv2d_gb300 as fv

    p = reference_params(Nx=96, Ny=80, gamma0=1.4, CFL=0.8)
    q = random_prim(80, 96, 5)
    q[17, 41, 3] = np.nan  # a NaN pressure: its sound speed and inverse dt are NaN
    s = fv.Simulation(p)
    s.set_prim(q)
    expect = np.array(s.compute_dt())
    o = Oracle(p)
    o.set_prim(q)
    assert bits_equal(expect, o.compute_dt())
    assert np.all(np.isfinite(expect))
    qd = torch.from_numpy(s.get_prim()).to("cuda")
    assert bool(torch.isnan(qd).any())
    out = torch.full((4,), -7.0, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    assert fv.compute_dt_noalloc(p, qd.data_ptr(), out.data_ptr(), stream.cuda_stream) == 0
    stream.synchronize()
    assert bits_equal(out.cpu().numpy(), expect)


def test_noalloc_rejects_grids_beyond_its_scratch(gpu_lib):
    import torch
    import fv2d_gb300 as fv

    out = torch.zeros(4, dtype=torch.float64, device="cuda")
    q = torch.zeros(8, dtype=torch.float64, device="cuda")
    big = reference_params(Nx=4097, Ny=4096)
    assert big.Nx * big.Ny > fv.NOALLOC_MAX_CELLS
    assert fv.compute_dt_noalloc(big, q.data_ptr(), out.data_ptr(), 0) == fv.ERR_SIZE
