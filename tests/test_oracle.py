"""The CPU oracle against the reference's published known answer, the
committed golden fixtures (produced by the reference's own headers) and,
where the reference checkout was available at build time, the reference
headers directly."""
import numpy as np
import pytest

from fv2d_testlib import (REF_OMP_SO, Oracle, RefSim, bits_equal, random_prim, ref_available, reference_params)
import golden.make_golden as G


def test_readme_blast_dt_log():
    """README.md:86-89: blast.ini prints dt_hyp 0.000521995 at t=0, then
    0.000480941 and 0.000459815 after 11 and 22 iterations."""
    p = reference_params(Nx=256, Ny=256, boundary_x=2, boundary_y=2, riemann_solver=1, reconstruction=0,
                         CFL=0.1, gamma0=1.4, tend=1.0)
    o = Oracle(p)
    o.init_problem("blast")
    hyp, dts = [], []
    t = 0.0
    for it in range(23):
        d = o.compute_dt()
        hyp.append(1.0 / d[1])
        dts.append(d[0])
        if it == 11:
            assert f"{t:.6g}" == "0.000551063"
        if it == 22:
            assert f"{t:.6g}" == "0.00106851"
        o.update(d[0])
        t += d[0]
    assert f"{hyp[0]:.6g}" == "0.000521995"
    assert f"{hyp[11]:.6g}" == "0.000480941"
    assert f"{hyp[22]:.6g}" == "0.000459815"
    gold = np.load(G.os.path.join(G.HERE, "blast_readme.npz"))
    assert bits_equal(np.array(dts), gold["dts"])


def test_sod_golden():
    gold = np.load(G.os.path.join(G.HERE, "sod_512x8.npz"))
    p = G.sod_params()
    o = Oracle(p)
    o.init_problem("sod_x")
    t, dts = o.run(p.tend, 100000)
    assert len(dts) == len(gold["dts"])
    assert bits_equal(dts, gold["dts"])
    assert bits_equal(o.get_prim(), gold["q"])
    assert t == float(gold["t"])


def test_combos_golden():
    gold = np.load(G.os.path.join(G.HERE, "combos.npz"))
    for n, c in enumerate(G.combo_list()):
        o = Oracle(reference_params(**G.COMBO_BASE, **c))
        o.set_prim(gold["q0"])
        for s in range(3):
            d = o.compute_dt()
            assert bits_equal(d[0], gold["dts"][n][s]), c
            o.update(d[0])
        assert bits_equal(o.get_prim(), gold["q"][n]), c


def test_problems_golden():
    gold = np.load(G.os.path.join(G.HERE, "problems.npz"))
    for n, name in enumerate(G.PROBLEM_NAMES):
        o = Oracle(reference_params(**G.PROBLEM_BASE))
        o.init_problem(name)
        for s in range(4):
            d = o.compute_dt()
            assert bits_equal(d[0], gold["dts"][n][s]), name
            o.update(d[0])
        assert bits_equal(o.get_prim(), gold["q"][n]), name


@pytest.mark.skipif(not ref_available(), reason="reference cross-check build (oracle/_ref) not present")
@pytest.mark.parametrize("seed", [3, 4])
def test_against_reference_headers(seed):
    """Random states, odd sizes, every combination, 4 iterations."""
    q0 = random_prim(9, 7, seed)
    for c in G.combo_list():
        p = reference_params(Nx=7, Ny=9, gamma0=1.4, CFL=0.6, **c)
        o, r = Oracle(p), RefSim(p)
        o.set_prim(q0)
        r.set_prim(q0)
        for _ in range(4):
            d = o.compute_dt()
            dr = r.compute_dt()
            assert bits_equal(d[0], dr), c
            o.update(d[0])
            r.update(dr)
        assert bits_equal(o.get_prim(), r.get_prim()), c
        assert bits_equal(o.get_cons(), r.get_cons()), c


@pytest.mark.skipif(not ref_available(), reason="reference cross-check build (oracle/_ref) not present")
@pytest.mark.parametrize("shape", [(2, 2), (2, 9), (9, 2)])
def test_smallest_grids_against_reference_headers(shape):
    """Grids of two cells along an axis: every ghost copies an interior cell
    (BoundaryConditions.h:22-71 with Nghosts = 2), every combination."""
    ny, nx = shape
    q0 = random_prim(ny, nx, 13)
    for c in G.combo_list():
        p = reference_params(Nx=nx, Ny=ny, gamma0=1.4, CFL=0.6, **c)
        o, r = Oracle(p), RefSim(p)
        o.set_prim(q0)
        r.set_prim(q0)
        for _ in range(3):
            d = o.compute_dt()
            dr = r.compute_dt()
            assert bits_equal(d[0], dr), c
            o.update(d[0])
            r.update(dr)
        assert bits_equal(o.get_prim(), r.get_prim()), c
        assert bits_equal(o.get_cons(), r.get_cons()), c


LONG_RUNS = [
    dict(riemann_solver=1, reconstruction=2, boundary_x=1, boundary_y=1),
    dict(riemann_solver=0, reconstruction=2, boundary_x=2, boundary_y=0, time_stepping=1),
    dict(riemann_solver=2, reconstruction=2, boundary_x=2, boundary_y=1, gravity_mode=1, gy=-0.5),
    dict(riemann_solver=0, reconstruction=2, boundary_x=2, boundary_y=1, gravity_mode=1, gy=-0.1, time_stepping=1,
         thermal_conductivity_active=1, kappa=1e-3, viscosity_active=1, mu=1e-3),
    dict(riemann_solver=1, reconstruction=0, boundary_x=0, boundary_y=2, well_balanced_flux_at_y_bc=1, gravity_mode=1,
         gy=-0.5),
]


@pytest.mark.skipif(not ref_available(), reason="reference cross-check build (oracle/_ref) not present")
@pytest.mark.parametrize("k", range(len(LONG_RUNS)))
def test_long_runs_against_reference_headers(k):
    """30 iterations on a 64 x 48 grid from random states: every dt and the
    final primitive and conservative fields."""
    q0 = random_prim(48, 64, 40 + k)
    p = reference_params(Nx=64, Ny=48, gamma0=1.4, CFL=0.6, **LONG_RUNS[k])
    o, r = Oracle(p), RefSim(p)
    o.set_prim(q0)
    r.set_prim(q0)
    for _ in range(30):
        d = o.compute_dt()
        dr = r.compute_dt()
        assert bits_equal(d[0], dr)
        o.update(d[0])
        r.update(dr)
    assert bits_equal(o.get_prim(), r.get_prim())
    assert bits_equal(o.get_cons(), r.get_cons())


@pytest.mark.skipif(not ref_available(), reason="reference cross-check build (oracle/_ref) not present")
def test_reference_reads_floats():
    """The reference's ini reader returns float-rounded reals (GetFloat)."""
    p = reference_params(Nx=8, Ny=8, gamma0=1.4, CFL=0.8)
    r = RefSim(p)
    assert r.param("gamma0") == float(np.float32(1.4))
    assert r.param("CFL") == float(np.float32(0.8))
    assert r.param("epsilon") == float(np.float32(1e-6))


def negative_case():
    """A strong two-sided expansion advanced with twice the CFL step: the
    update drives the central densities negative (used by the GPU tests too)."""
    q = np.ones((6, 6, 4))
    q[..., 2] = 0.0
    q[..., 3] = 1e-3
    q[:, :3, 1] = -30.0
    q[:, 3:, 1] = 30.0
    p = reference_params(Nx=6, Ny=6, gamma0=1.4, CFL=0.9, boundary_x=1, boundary_y=1)
    return p, q


def test_negative_reset_counters():
    """checkNegatives (SimInfo.h:602-646): negative densities are reset to
    epsilon_reset_negative and counted."""
    p, q = negative_case()
    o = Oracle(p)
    o.set_prim(q)
    d = o.compute_dt()
    o.update(2.0 * d[0])
    c = o.counters()
    assert c[0] == 12 and c[2] == 0
    assert (o.get_prim()[..., 0] > 0).all()


@pytest.mark.parametrize("recon", [2, 3])  # PLM; MUSCL-Hancock (the benchmark's CPU set-up, no reference counterpart)
def test_sod_converges_to_the_exact_riemann_solution(recon):
    """Physics check of the scheme the oracle restates (and the GPU path
    reproduces bit for bit): the Sod problem of the benchmark set-up against
    the exact Riemann solution (tests/exact_riemann.py), in L1 for rho, u
    and p, with the error shrinking as the grid is refined."""
    import exact_riemann as ER
    g = float(np.float32(1.4))
    errs = {}
    for nx in (128, 512):
        p = reference_params(Nx=nx, Ny=8, xmin=0.0, xmax=1.0, ymin=0.0, ymax=1.0 / 64, gamma0=1.4,
                             reconstruction=recon, riemann_solver=1, CFL=0.8, boundary_x=0, boundary_y=2, tend=0.2)
        o = Oracle(p)
        o.init_problem("sod_x")
        t, _ = o.run(p.tend, 100000)
        q = o.get_prim()
        assert np.all(q == q[:1]), "rows of the y-uniform problem differ"
        x = (np.arange(nx) + 0.5) / nx
        rho, u, pr = ER.profile((1.0, 0.0, 1.0), (0.125, 0.0, 0.1), g, x, 0.5, t)
        errs[nx] = [float(np.mean(np.abs(q[0, :, k] - ex))) for k, ex in ((0, rho), (1, u), (3, pr))]
    print(errs)
    assert all(e < 1e-2 for e in errs[512]), errs
    assert all(errs[512][k] < 0.5 * errs[128][k] for k in range(3)), errs


def test_restart_is_not_bit_exact_against_continuing():
    """A restart rebuilds U = primToCons(Q) from the stored primitives
    (IOManager.h:358-379, then primToCons as at start-up); consToPrim then
    primToCons does not return every conservative value bit for bit, so a
    restarted run differs from the continued one at rounding level.  (The GPU
    path's restart is compared with the oracle's restart, bitwise, in the
    driver tests.)"""
    p = reference_params(Nx=128, Ny=128, gamma0=1.4, reconstruction=2, riemann_solver=1, CFL=0.6,
                         boundary_x=2, boundary_y=2)
    a, b = Oracle(p), Oracle(p)
    a.init_problem("kh_step")
    b.init_problem("kh_step")
    for _ in range(10):
        for o in (a, b):
            o.update(o.compute_dt()[0])
    u_before = b.get_cons()
    b.set_prim(b.get_prim())  # what a restart from a snapshot of this state does
    changed = np.sum(u_before != b.get_cons())
    assert 0 < changed < u_before.size // 4
    for _ in range(30):
        for o in (a, b):
            o.update(o.compute_dt()[0])
    qa, qb = a.get_prim(), b.get_prim()
    assert not bits_equal(qa, qb)
    assert np.max(np.abs(qa - qb) / np.abs(qa).max(axis=(0, 1))) < 1e-9


@pytest.mark.skipif(not ref_available(REF_OMP_SO), reason="OpenMP build of the reference headers not present")
def test_openmp_build_of_the_reference_headers_matches_the_oracle():
    """The build used to time the reference's own step code on the host
    cores (OpenMP over rows) gives the oracle's bits: its timing is a timing
    of the same arithmetic."""
    q0 = random_prim(64, 96, 7)
    for c in LONG_RUNS[:3]:
        p = reference_params(Nx=96, Ny=64, gamma0=1.4, CFL=0.6, **c)
        o, r = Oracle(p), RefSim(p, lib_path=REF_OMP_SO)
        o.set_prim(q0)
        r.set_prim(q0)
        for _ in range(10):
            d = o.compute_dt()
            dr = r.compute_dt()
            assert bits_equal(d[0], dr)
            o.update(d[0])
            r.update(dr)
        assert bits_equal(o.get_prim(), r.get_prim())


def test_round_cons_f32_hook_rounds_the_stored_offsets():
    """The accuracy-floor hook: every conservative value becomes the binary32
    rounding of its offset from the background, plus the background; the
    primitives are rebuilt from it."""
    import ctypes as C
    from fv2d_testlib import oracle_lib
    lib = oracle_lib()
    lib.fv2d_oracle_round_cons_f32.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
    p = reference_params(Nx=24, Ny=16, gamma0=1.4)
    q = random_prim(16, 24, 3)
    for bg in (None, np.array([1.3, 0.0, 0.0, 2.7])):
        o = Oracle(p)
        o.set_prim(q)
        u0 = o.get_cons()
        ptr = None if bg is None else bg.ctypes.data_as(C.POINTER(C.c_double))
        assert lib.fv2d_oracle_round_cons_f32(o.h, ptr) == 0
        b = np.zeros(4) if bg is None else bg
        expect = (u0 - b).astype(np.float32).astype(np.float64) + b
        assert bits_equal(o.get_cons(), expect)
        u = o.get_cons()
        qq = o.get_prim()
        assert np.allclose(qq[..., 1], u[..., 1] / u[..., 0], rtol=1e-15)
        assert not bits_equal(o.get_cons(), u0)


def test_accuracy_floor_background_matches_the_service_rule():
    """tests/accuracy_floor.py restates the service's background choice:
    upper medians of rho and E over the cells (sy/2 + k sy, sx/2 + l sx),
    sx = max(1, Nx / 64), rounded to binary32."""
    import accuracy_floor as AF
    u = np.zeros((100, 130, 4))
    u[..., 0] = np.arange(100 * 130).reshape(100, 130)
    u[..., 3] = -u[..., 0]
    bg = AF.service_background(u, 130, 100)
    sub = u[0::1, 1::2]  # sy = 1, sx = 2
    assert bg[0] == float(np.float32(np.sort(sub[..., 0].ravel())[sub[..., 0].size // 2]))
    assert bg[3] == float(np.float32(np.sort(sub[..., 3].ravel())[sub[..., 3].size // 2]))
    assert bg[1] == bg[2] == 0.0
