"""GPU parity of the plain FP64 path, through the C-ABI.

The bar is bit-identical binary64 results: every dt and every primitive
value equal to the reference's (golden fixtures from the reference's own
headers) and to the oracle (same seeded inputs), including odd grid sizes
that cut tiles, every switch combination and the device-driven loop.  At the
full benchmark size (2048^2) the GPU is compared bitwise with the OpenMP
oracle for a few iterations, and checked for exact mass conservation
properties and run-to-run determinism.
"""
import numpy as np
import pytest

import golden.make_golden as G
from fv2d_testlib import Oracle, bits_equal, random_prim, reference_params
from test_oracle import negative_case

pytestmark = pytest.mark.gpu


def gpu_sim(p):
    from fv2d_gb300 import Simulation
    return Simulation(p)


def test_combos_match_reference_fixtures(gpu_lib):
    gold = np.load(G.os.path.join(G.HERE, "combos.npz"))
    for n, c in enumerate(G.combo_list()):
        s = gpu_sim(reference_params(**G.COMBO_BASE, **c))
        s.set_prim(gold["q0"])
        for k in range(3):
            dt = s.compute_dt()[0]
            assert bits_equal(dt, gold["dts"][n][k]), (c, k, dt, gold["dts"][n][k])
            s.update(dt)
        assert bits_equal(s.get_prim(), gold["q"][n]), c
        s.close()


def test_problems_match_reference_fixtures(gpu_lib):
    gold = np.load(G.os.path.join(G.HERE, "problems.npz"))
    for n, name in enumerate(G.PROBLEM_NAMES):
        s = gpu_sim(reference_params(**G.PROBLEM_BASE))
        s.init_problem(name)
        for k in range(4):
            dt = s.compute_dt()[0]
            assert bits_equal(dt, gold["dts"][n][k]), name
            s.update(dt)
        assert bits_equal(s.get_prim(), gold["q"][n]), name
        s.close()


def test_sod_512x8_device_loop_matches_reference(gpu_lib):
    """BASELINE Sod set-up run to t = 0.2 by the device-driven loop: the dt
    sequence (per-iteration log) and the final primitives are the reference's."""
    gold = np.load(G.os.path.join(G.HERE, "sod_512x8.npz"))
    p = G.sod_params()
    s = gpu_sim(p)
    s.init_problem("sod_x")
    t, n, status = s.advance(100000, p.tend)
    from fv2d_gb300 import RUN_DONE
    assert status == RUN_DONE
    assert n == len(gold["dts"])
    log = s.step_log()
    assert bits_equal(log[:, 1], gold["dts"])
    assert t == float(gold["t"])
    assert bits_equal(s.get_prim(), gold["q"])


def test_sod_granular_calls_match_device_loop(gpu_lib):
    p = G.sod_params()
    a, b = gpu_sim(p), gpu_sim(p)
    a.init_problem("sod_x")
    b.init_problem("sod_x")
    t = 0.0
    for _ in range(50):
        dt = a.compute_dt()[0]
        a.update(dt)
        t += dt
    tb, n, _ = b.advance(50, 10.0)
    assert n == 50 and tb == t
    assert bits_equal(a.get_prim(), b.get_prim())
    assert bits_equal(a.get_cons(), b.get_cons())


@pytest.mark.parametrize("shape", [(17, 33), (40, 65), (37, 100), (5, 3), (2, 2), (2, 9), (9, 2)])
def test_odd_sizes_match_oracle(gpu_lib, shape):
    ny, nx = shape
    q0 = random_prim(ny, nx, 11 + nx)
    for c in G.combo_list()[::7]:
        p = reference_params(Nx=nx, Ny=ny, gamma0=1.4, CFL=0.6, **c)
        o, s = Oracle(p), gpu_sim(p)
        o.set_prim(q0)
        s.set_prim(q0)
        for _ in range(3):
            d = o.compute_dt()
            assert bits_equal(s.compute_dt()[0], d[0]), c
            o.update(d[0])
            s.update(d[0])
        assert bits_equal(s.get_prim(), o.get_prim()), c
        assert bits_equal(s.get_cons(), o.get_cons()), c
        s.close()


def test_sod_benchmark_with_muscl_hancock_matches_oracle(gpu_lib):
    """The CPU-runnable benchmark set-up as specified -- Sod 512x8, PLM slopes
    with the MUSCL-Hancock half-step, HLLC, CFL 0.8, outflow in x, periodic
    in y, to t = 0.2 -- through the device loop, bitwise against the oracle
    (every dt, t, the fields)."""
    p = reference_params(Nx=512, Ny=8, xmin=0.0, xmax=1.0, ymin=0.0, ymax=1.0 / 64, gamma0=1.4, reconstruction=3,
                         riemann_solver=1, CFL=0.8, boundary_x=0, boundary_y=2, tend=0.2)
    o, s = Oracle(p), gpu_sim(p)
    o.init_problem("sod_x")
    s.init_problem("sod_x")
    dts, t_ref = [], 0.0
    while t_ref + p.epsilon < p.tend:
        d = o.compute_dt()
        dts.append(d[0])
        o.update(d[0])
        t_ref += d[0]
    t, n, _ = s.advance(100000, p.tend)
    assert n == len(dts) and t == t_ref
    assert bits_equal(s.step_log(4096)[:, 1], np.array(dts))
    assert bits_equal(s.get_prim(), o.get_prim())


def test_muscl_hancock_extension_matches_oracle(gpu_lib):
    q0 = random_prim(19, 37, 5, smooth=True)
    for rs in (0, 1, 2):
        for bc in (0, 1, 2):
            p = reference_params(Nx=37, Ny=19, gamma0=1.4, CFL=0.5, reconstruction=3, riemann_solver=rs,
                                 boundary_x=bc, boundary_y=(bc + 1) % 3)
            o, s = Oracle(p), gpu_sim(p)
            o.set_prim(q0)
            s.set_prim(q0)
            for _ in range(4):
                d = o.compute_dt()
                o.update(d[0])
                s.update(d[0])
            assert bits_equal(s.get_prim(), o.get_prim()), (rs, bc)
            s.close()


@pytest.mark.parametrize("name", ["sedov", "kh_step", "rt_hydrostatic", "H84", "C91", "gresho_vortex", "blast"])
def test_initial_conditions_match_oracle(gpu_lib, name):
    kw = dict(Nx=48, Ny=40, gamma0=1.4, CFL=0.5, reconstruction=2)
    if name == "rt_hydrostatic":
        kw.update(gravity_mode=1, gy=-0.1, riemann_solver=0, boundary_x=2, xmax=0.5, ymax=1.5)
    if name in ("H84", "C91"):
        kw.update(ymin=1.0, ymax=2.0, gravity_mode=1, gy=-1.0)
    p = reference_params(**kw)
    o, s = Oracle(p), gpu_sim(p)
    o.init_problem(name)
    s.init_problem(name)
    assert bits_equal(s.get_prim(), o.get_prim())
    for _ in range(3):
        d = o.compute_dt()
        assert bits_equal(s.compute_dt()[0], d[0])
        o.update(d[0])
        s.update(d[0])
    assert bits_equal(s.get_prim(), o.get_prim())


def test_negative_counters_match_oracle(gpu_lib):
    p, q = negative_case()
    o, s = Oracle(p), gpu_sim(p)
    o.set_prim(q)
    s.set_prim(q)
    dt = o.compute_dt()[0]
    o.update(2 * dt)
    s.update(2 * dt)
    assert s.counters() == o.counters() == [12, 0, 0]
    assert bits_equal(s.get_prim(), o.get_prim())


def test_device_loop_stops_for_snapshots(gpu_lib):
    """main.cpp:62-84: the save test happens before dt at each iteration and
    at most once per iteration."""
    p = G.sod_params()
    p.tend = 0.05
    s = gpu_sim(p)
    s.init_problem("sod_x")
    o = Oracle(p)
    o.init_problem("sod_x")
    save_freq, next_save, t, ite = 0.01, 0.0, 0.0, 0
    saves_host = []
    while t + p.epsilon < p.tend:  # reference loop on the oracle
        if t + p.epsilon > next_save:
            saves_host.append(t)
            next_save += save_freq
        d = o.compute_dt()
        o.update(d[0])
        t += d[0]
        ite += 1
    saves_dev, next_save, skip = [], 0.0, False
    while True:
        td, n, status = s.advance(1000000, p.tend, next_save, skip)
        from fv2d_gb300 import RUN_DONE, RUN_SAVE
        if status == RUN_SAVE:
            saves_dev.append(td)
            next_save += save_freq
            skip = True
            continue
        assert status == RUN_DONE
        break
    assert saves_dev == saves_host
    assert td == t
    assert bits_equal(s.get_prim(), o.get_prim())


@pytest.mark.slow
def test_full_size_sedov_matches_oracle(gpu_lib):
    """Sedov 2048^2 (the benchmark grid): bitwise against the OpenMP oracle
    for 3 iterations, then conservation and determinism over 40 more."""
    p = reference_params(Nx=2048, Ny=2048, gamma0=1.4, reconstruction=2, riemann_solver=1, CFL=0.8,
                         boundary_x=1, boundary_y=1)
    o, s = Oracle(p), gpu_sim(p)
    o.init_problem("sedov")
    s.init_problem("sedov")
    for _ in range(3):
        d = o.compute_dt()
        assert bits_equal(s.compute_dt()[0], d[0])
        o.update(d[0])
        s.update(d[0])
    assert bits_equal(s.get_prim(), o.get_prim())
    del o
    u0 = s.get_cons()
    s.advance(40, 1e9)
    u1 = s.get_cons()
    # reflecting walls: mass and energy are conserved to summation rounding
    for k in (0, 3):
        a, b = np.sum(u0[..., k], dtype=np.float64), np.sum(u1[..., k], dtype=np.float64)
        assert abs(b - a) <= 1e-11 * abs(a), k
    # run-to-run determinism
    s2 = gpu_sim(p)
    s2.init_problem("sedov")
    for _ in range(3):
        s2.update(s2.compute_dt()[0])
    s2.advance(40, 1e9)
    assert bits_equal(s2.get_cons(), u1)


@pytest.mark.slow
def test_sedov_benchmark_run_matches_oracle_after_1000_steps(gpu_lib):
    """The benchmark run itself -- Sedov 2048^2, PLM + HLLC, CFL 0.8,
    reflecting walls, 1000 iterations from the initial condition through
    the device-driven loop -- bitwise against the oracle (OpenMP over the
    host cores, ~30 s on 16 cores): every dt and the final fields."""
    p = reference_params(Nx=2048, Ny=2048, gamma0=1.4, reconstruction=2, riemann_solver=1, CFL=0.8,
                         boundary_x=1, boundary_y=1)
    o, s = Oracle(p), gpu_sim(p)
    o.init_problem("sedov")
    s.init_problem("sedov")
    dts = []
    for _ in range(1000):
        d = o.compute_dt()
        dts.append(d[0])
        o.update(d[0])
    t, n, _ = s.advance(1000, 1e30)
    assert n == 1000
    log = s.step_log(1000)
    assert len(log) == 1000 and bits_equal(log[:, 1], np.array(dts))
    t_ref = 0.0
    for d in dts:  # t += dt in binary64, in order (main.cpp:83)
        t_ref += d
    assert t == t_ref
    assert bits_equal(s.get_prim(), o.get_prim())
    assert o.counters() == s.counters()


FULL_SIZE = {
    # KH 4096^2, CFL 0.7, periodic: mass, both momenta and energy are conserved
    "kh_4096": ("kh_step", dict(Nx=4096, Ny=4096, gamma0=1.4, reconstruction=2, riemann_solver=1, CFL=0.7,
                                boundary_x=2, boundary_y=2), (0, 1, 2, 3)),
    # RT 1024x3072 (HLL, gravity, conduction, viscosity), periodic in x, reflecting in y: mass is conserved
    "rt_1024x3072": ("rt_hydrostatic", dict(Nx=1024, Ny=3072, xmax=0.5, ymax=1.5, gamma0=1.4, reconstruction=2,
                                            riemann_solver=0, CFL=0.8, boundary_x=2, boundary_y=1, gravity_mode=1,
                                            gy=-0.1, thermal_conductivity_active=1, kappa=1e-4,
                                            viscosity_active=1, mu=1e-4), (0,)),
}


@pytest.mark.slow
@pytest.mark.parametrize("case", sorted(FULL_SIZE))
def test_full_size_kh_and_rt_match_oracle(gpu_lib, case):
    """The other two benchmark set-ups at their full sizes: bitwise against
    the oracle for 3 iterations, then the conserved sums over 20 more."""
    problem, kw, conserved = FULL_SIZE[case]
    p = reference_params(**kw)
    o, s = Oracle(p), gpu_sim(p)
    o.init_problem(problem)
    s.init_problem(problem)
    for _ in range(3):
        d = o.compute_dt()
        assert bits_equal(s.compute_dt()[0], d[0])
        o.update(d[0])
        s.update(d[0])
    assert bits_equal(s.get_prim(), o.get_prim())
    assert o.counters() == s.counters()
    del o
    u0 = s.get_cons()
    s.advance(20, 1e9)
    u1 = s.get_cons()
    for k in conserved:
        a, b = np.sum(u0[..., k], dtype=np.float64), np.sum(u1[..., k], dtype=np.float64)
        scale = np.sum(np.abs(u0[..., k]), dtype=np.float64)
        assert abs(b - a) <= 1e-10 * scale, (k, a, b)


def test_page_locked_input_and_host_mirror_match_pageable_path(gpu_lib):
    """set_prim from page-locked memory (read by the set-up kernel over the
    host link) and the host mirror written by the step kernel give the same
    bits as the staged copies, for Euler and RK2 and tiles cut by odd sizes;
    after set_prim the mirror is stale and get_prim copies again."""
    torch = pytest.importorskip("torch")
    from fv2d_gb300 import Fv2dError
    ny, nx = 40, 65
    q0 = random_prim(ny, nx, 5)
    pin_in = torch.from_numpy(q0.copy()).pin_memory()
    pin_out = torch.zeros((ny, nx, 4), dtype=torch.float64).pin_memory()
    for c in G.combo_list()[::19]:
        p = reference_params(Nx=nx, Ny=ny, gamma0=1.4, CFL=0.6, **c)
        a, b, o = gpu_sim(p), gpu_sim(p), Oracle(p)
        with pytest.raises(Fv2dError):
            a.set_host_mirror(q0.ctypes.data)  # pageable memory is refused
        a.set_host_mirror(pin_out.data_ptr())
        a.set_prim_ptr(pin_in.data_ptr())
        b.set_prim(q0)
        o.set_prim(q0)
        for _ in range(3):
            d = o.compute_dt()
            assert bits_equal(a.compute_dt()[0], d[0]) and bits_equal(b.compute_dt()[0], d[0]), c
            a.update(d[0])
            b.update(d[0])
            o.update(d[0])
            a.get_prim_ptr(pin_out.data_ptr())
            ref = o.get_prim()
            assert bits_equal(pin_out.numpy(), ref), c
            assert bits_equal(b.get_prim(), ref), c
        a.set_prim_ptr(pin_in.data_ptr())
        a.get_prim_ptr(pin_out.data_ptr())
        assert bits_equal(pin_out.numpy(), q0), c
        a.set_host_mirror(0)
        a.close()
        b.close()


def test_page_locked_rounds_match_oracle(gpu_lib):
    """Rounds of set_prim from page-locked memory (read by the set-up kernel),
    compute_dt, update writing the host mirror and get_prim on the mirror --
    the end-to-end benchmark's call sequence -- give the oracle's bits for
    every Euler combination of PCM / PCM_WB / PLM, HLL / HLLC, boundaries
    and gravity, on a grid that cuts tiles."""
    torch = pytest.importorskip("torch")
    ny, nx = 37, 50
    q0 = random_prim(ny, nx, 9)
    pin_in = torch.from_numpy(q0.copy()).pin_memory()
    pin_out = torch.zeros((ny, nx, 4), dtype=torch.float64).pin_memory()
    combos = [c for c in G.combo_list() if c.get("time_stepping", 0) == 0 and c.get("riemann_solver", 1) in (0, 1)
              and not c.get("thermal_conductivity_active") and not c.get("viscosity_active")
              and not c.get("well_balanced_flux_at_y_bc")]
    assert len(combos) >= 18
    for c in combos:
        p = reference_params(Nx=nx, Ny=ny, gamma0=1.4, CFL=0.6, **c)
        s, o = gpu_sim(p), Oracle(p)
        s.set_host_mirror(pin_out.data_ptr())
        q = q0
        for _ in range(3):
            pin_in.numpy()[...] = q
            s.set_prim_ptr(pin_in.data_ptr())
            o.set_prim(q)
            d = o.compute_dt()
            assert bits_equal(s.compute_dt()[0], d[0]), c
            s.update(d[0])
            o.update(d[0])
            s.get_prim_ptr(pin_out.data_ptr())
            q = o.get_prim()
            assert bits_equal(pin_out.numpy(), q), c
            assert bits_equal(s.get_cons(), o.get_cons()), c
        s.set_host_mirror(0)
        s.close()


def test_prefetched_input_rounds_match_oracle(gpu_lib):
    """The pipelined end-to-end sequence: the next input prefetched over the
    host link while the current step runs, then set_prim of that pointer
    builds the state from the staging buffer -- the oracle's bits, round
    after round, with a new input each round.  A prefetch dropped by another
    use of the staging buffer (get_cons, a pageable set_prim) is read again
    from the host array; pageable memory cannot be prefetched."""
    torch = pytest.importorskip("torch")
    from fv2d_gb300 import Fv2dError
    ny, nx = 37, 50
    inputs = [random_prim(ny, nx, 30 + k) for k in range(4)]
    pin_in = torch.zeros((ny, nx, 4), dtype=torch.float64).pin_memory()
    pin_out = torch.zeros((ny, nx, 4), dtype=torch.float64).pin_memory()
    for c in G.combo_list()[::23]:
        p = reference_params(Nx=nx, Ny=ny, gamma0=1.4, CFL=0.6, **c)
        s, o = gpu_sim(p), Oracle(p)
        with pytest.raises(Fv2dError):
            s.prefetch_prim_ptr(inputs[0].ctypes.data)
        s.set_host_mirror(pin_out.data_ptr())
        pin_in.numpy()[...] = inputs[0]
        s.set_prim_ptr(pin_in.data_ptr())
        for k in range(3):
            o.set_prim(inputs[k])
            d = o.compute_dt()
            assert bits_equal(s.compute_dt()[0], d[0]), c
            s.update(d[0])
            o.update(d[0])
            s.get_prim_ptr(pin_out.data_ptr())
            assert bits_equal(pin_out.numpy(), o.get_prim()), (c, k)
            pin_in.numpy()[...] = inputs[k + 1]  # the caller fills the next input, then prefetches it
            s.prefetch_prim_ptr(pin_in.data_ptr())
            if k == 1:
                s.get_cons()  # uses the staging buffer: the prefetch is dropped
            s.set_prim_ptr(pin_in.data_ptr())
            o.set_prim(inputs[k + 1])
            assert bits_equal(s.get_cons(), o.get_cons()), (c, k)
        # a prefetch followed by a set_prim of another (pageable) array
        s.prefetch_prim_ptr(pin_in.data_ptr())
        s.set_prim(inputs[0])
        s.get_prim_ptr(pin_out.data_ptr())
        assert bits_equal(pin_out.numpy(), inputs[0]), c
        s.set_host_mirror(0)
        s.close()
