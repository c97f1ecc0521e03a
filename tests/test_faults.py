"""Failure handling that faults, traps or hangs no GPU.

* The device-side wait guard: a bounded wait on a barrier that nothing
  completes returns with its error bit set, and the context keeps working.
* A NaN planted in the initial data (on the host) propagates, and is counted
  by checkNegatives (SimInfo.h:602-646), exactly as in the oracle.
* In the served loop, a request whose state turns NaN fails with
  FV2D_ERR_NUMERIC while the requests batched with it finish with the same
  results as alone; a request that can never fit the memory budget is refused
  at submission.
* A failure of the served worker's CUDA stream, simulated on the host by the
  library's test hook: every resident and queued request completes with
  FV2D_ERR_CUDA, drain returns that code, and later submissions are refused.
"""
import numpy as np
import pytest

from fv2d_gb300._abi import ERR_NUMERIC
from fv2d_testlib import Oracle, bits_equal, random_prim, reference_params

pytestmark = pytest.mark.gpu


def test_bounded_wait_times_out_and_the_context_stays_usable(gpu_lib):
    import fv2d_gb300 as fv
    assert fv.selftest_wait_timeout(1000) == 1  # DEVERR_TMA_TIMEOUT
    p = reference_params(Nx=32, Ny=16, gamma0=1.4, CFL=0.6, reconstruction=fv.PLM, riemann_solver=fv.HLLC)
    q0 = random_prim(16, 32, 4)
    s, o = fv.Simulation(p), Oracle(p)
    s.set_prim(q0)
    o.set_prim(q0)
    d = o.compute_dt()
    s.update(d[0])
    o.update(d[0])
    assert bits_equal(s.get_prim(), o.get_prim())
    s.close()


@pytest.mark.parametrize("field", [0, 3])
def test_nan_in_the_initial_state_is_counted_like_the_oracle(gpu_lib, field):
    import fv2d_gb300 as fv
    ny, nx = 17, 33
    q0 = random_prim(ny, nx, 21)
    q0[6, 11, field] = np.nan
    p = reference_params(Nx=nx, Ny=ny, gamma0=1.4, CFL=0.6, reconstruction=fv.PLM, riemann_solver=fv.HLLC,
                         boundary_x=fv.BC_PERIODIC, boundary_y=fv.BC_REFLECTING)
    s, o = fv.Simulation(p), Oracle(p)
    s.set_prim(q0)
    o.set_prim(q0)
    for _ in range(3):
        d = o.compute_dt()
        assert bits_equal(s.compute_dt()[0], d[0])
        s.update(d[0])
        o.update(d[0])
        assert s.counters() == o.counters()
    assert o.counters()[2] > 0  # NaNs seen by checkNegatives
    assert bits_equal(s.get_prim(), o.get_prim())
    s.close()


def _params(N, **kw):
    import fv2d_gb300 as fv
    f = fv.as_float32
    base = dict(Nx=N, Ny=N, gamma0=f(1.4), CFL=f(0.8), reconstruction=fv.PLM, riemann_solver=fv.HLLC,
                boundary_x=fv.BC_REFLECTING, boundary_y=fv.BC_REFLECTING)
    base.update(kw)
    return fv.default_params(**base)


@pytest.mark.parametrize("tile", [None, "28/128x4/march"])
def test_served_nan_request_fails_alone(gpu_lib, tile):
    import fv2d_gb300 as fv
    from fv2d_gb300.serve import Server
    good = [("sedov", _params(128), 40), ("sedov", _params(192), 30),
            ("kh_step", _params(96, boundary_x=fv.BC_PERIODIC, boundary_y=fv.BC_PERIODIC, seed=3), 35)]
    bad = ("sod_x", _params(128, boundary_x=fv.BC_ABSORBING, boundary_y=fv.BC_PERIODIC, sod_rho_right=float("nan")),
           50)
    alone = []
    with Server(budget_bytes=2e9, autotune=False, tile_config=tile) as s:
        for pb, p, n in good:
            rid = s.submit(pb, p, n)
            assert s.drain(120) == 0
            res = {r.id: r for r in s.poll()}
            assert res[rid].status == 0
            alone.append(s.get_prim(rid))
    with Server(budget_bytes=2e9, autotune=False, tile_config=tile) as s:
        ids = [s.submit(pb, p, n) for pb, p, n in good[:2]]
        bid = s.submit(*bad)
        ids.append(s.submit(*good[2]))
        assert s.drain(120) == 0
        res = {r.id: r for r in s.poll()}
        assert res[bid].status == ERR_NUMERIC and res[bid].steps < bad[2]
        for k, rid in enumerate(ids):
            assert res[rid].status == 0 and res[rid].steps == good[k][2]
            assert bits_equal(s.get_prim(rid), alone[k])


def test_served_refuses_a_request_larger_than_the_budget(gpu_lib):
    from fv2d_gb300.serve import Server
    with Server(budget_bytes=1e6, autotune=False) as s:  # a 256^2 state pair needs 2.4 MB
        with pytest.raises(ValueError):
            s.submit("sedov", _params(256), 10)


def test_served_worker_failure_fails_every_request_and_refuses_new_ones(gpu_lib):
    import time
    from fv2d_gb300._abi import ERR_CUDA
    from fv2d_gb300.serve import Server
    # the budget holds one 128^2 state pair (0.68 MB): one request resident, two queued
    with Server(budget_bytes=1e6, autotune=False) as s:
        ids = [s.submit("sedov", _params(128), 1 << 30) for _ in range(3)]
        deadline = time.time() + 60
        while time.time() < deadline:
            st = s.stats()
            if st.admitted == 1 and st.queued == 2:
                break
            time.sleep(0.01)
        assert st.admitted == 1 and st.queued == 2
        assert s.last_error() == ""
        s.inject_fault()
        assert s.drain(60) == ERR_CUDA
        res = {r.id: r for r in s.poll()}
        assert sorted(res) == sorted(ids)
        assert all(r.status == ERR_CUDA for r in res.values())
        st = s.stats()
        assert (st.failed, st.completed, st.active, st.queued) == (3, 0, 0, 0)
        assert "simulated" in s.last_error()
        with pytest.raises(RuntimeError):
            s.submit("sedov", _params(128), 10)
        with pytest.raises(KeyError):
            s.get_prim(ids[0])
