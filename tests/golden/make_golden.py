"""Generates the golden fixtures in tests/golden/ by running the reference's
own hot-path headers (compiled from the reference checkout by
oracle/ref_check/build.sh into oracle/_ref/libfv2d_ref.so, against a serial
stand-in for the Kokkos/inih entry points they use).

Fixtures (numpy .npz, float64):
  sod_512x8.npz         BASELINE Sod set-up: 512x8 on [0,1]x[0,1/64], gamma 1.4,
                        PLM/minmod, HLLC, CFL 0.8, absorbing x, periodic y,
                        run to t = 0.2: dt sequence, final primitives.
  blast_readme.npz      settings/blast.ini (256x256): dt of the first 23
                        iterations, the README's published log (README.md:86-89)
                        being iterations 0, 11 and 22.
  combos.npz            random 14x10 states x every (solver, reconstruction,
                        time stepping, boundary) combination and the physics
                        switches: initial state, dt of each of 3 iterations and
                        final primitives.
  problems.npz          every reference initial condition on 16x16 after 4
                        PLM/HLLC iterations.

Run: python tests/golden/make_golden.py   (needs oracle/_ref built)
"""
import itertools
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, os.path.dirname(HERE))

from fv2d_testlib import RefSim, random_prim, reference_params  # noqa: E402


def sod_params():
    return reference_params(Nx=512, Ny=8, xmin=0.0, xmax=1.0, ymin=0.0, ymax=1.0 / 64, gamma0=1.4,
                            reconstruction=2, riemann_solver=1, CFL=0.8, boundary_x=0, boundary_y=2, tend=0.2)


def combo_list():
    out = []
    for rs, rec, ts, bcx, bcy in itertools.product([0, 1, 2], [0, 1, 2], [0, 1], [0, 1, 2], [0, 1, 2]):
        out.append(dict(riemann_solver=rs, reconstruction=rec, time_stepping=ts, boundary_x=bcx, boundary_y=bcy))
    phys = [
        dict(gravity_mode=1, gx=0.05, gy=-0.1),
        dict(gravity_mode=2, hot_bubble_g0=0.3),
        dict(thermal_conductivity_active=1, kappa=1e-2),
        dict(viscosity_active=1, mu=1e-2),
        dict(thermal_conductivity_active=1, kappa=1e-2, bctc_ymin=1, bctc_ymax=2, bctc_ymin_value=1.5,
             bctc_ymax_value=0.3),
        dict(gravity_mode=1, gy=-0.5, well_balanced_flux_at_y_bc=1),
        dict(gravity_mode=1, gy=-0.5, riemann_solver=2, reconstruction=2),
        dict(gravity_mode=1, gy=-0.1, thermal_conductivity_active=1, kappa=1e-3, viscosity_active=1, mu=1e-3,
             riemann_solver=0, reconstruction=2, time_stepping=1),
    ]
    for ph in phys:
        for rec in (0, 2):
            d = dict(ph)
            d.setdefault("reconstruction", rec)
            out.append(d)
    return out


COMBO_BASE = dict(Nx=14, Ny=10, gamma0=1.4, CFL=0.5)
PROBLEM_NAMES = ["sod_x", "sod_y", "blast", "rayleigh-taylor", "diffusion", "kelvin_helmholtz", "gresho_vortex"]
PROBLEM_BASE = dict(Nx=16, Ny=16, gamma0=1.4, CFL=0.4, reconstruction=2, boundary_x=2, boundary_y=2)


def main():
    # Sod
    p = sod_params()
    r = RefSim(p, "sod_x")
    r.init()
    t, dts = 0.0, []
    while t + p.epsilon < p.tend:
        dt = r.compute_dt()
        dts.append(dt)
        r.update(dt)
        t += dt
    np.savez_compressed(os.path.join(HERE, "sod_512x8.npz"), dts=np.array(dts), t=t, q=r.get_prim())
    print("sod", len(dts), "iterations, t =", t)

    # blast.ini known answer
    pb = reference_params(Nx=256, Ny=256, xmin=0.0, xmax=1.0, ymin=0.0, ymax=1.0, tend=1.0, save_freq=0.01,
                          boundary_x=2, boundary_y=2, riemann_solver=1, reconstruction=0, CFL=0.1, gamma0=1.4)
    r = RefSim(pb, "blast")
    r.init()
    dts = []
    for _ in range(23):
        dt = r.compute_dt()
        dts.append(dt)
        r.update(dt)
    np.savez_compressed(os.path.join(HERE, "blast_readme.npz"), dts=np.array(dts))

    # switch combinations on random data
    combos = combo_list()
    q0 = random_prim(COMBO_BASE["Ny"], COMBO_BASE["Nx"], 1)
    dts, qs = [], []
    for c in combos:
        pc = reference_params(**COMBO_BASE, **c)
        r = RefSim(pc)
        r.set_prim(q0)
        d = []
        for _ in range(3):
            dt = r.compute_dt()
            d.append(dt)
            r.update(dt)
        dts.append(d)
        qs.append(r.get_prim())
    np.savez_compressed(os.path.join(HERE, "combos.npz"), q0=q0, dts=np.array(dts), q=np.array(qs))
    print("combos", len(combos))

    # reference problems
    qs, dts = [], []
    for name in PROBLEM_NAMES:
        pp = reference_params(**PROBLEM_BASE)
        r = RefSim(pp, name)
        r.init()
        d = []
        for _ in range(4):
            dt = r.compute_dt()
            d.append(dt)
            r.update(dt)
        dts.append(d)
        qs.append(r.get_prim())
    np.savez_compressed(os.path.join(HERE, "problems.npz"), dts=np.array(dts), q=np.array(qs))
    print("problems", len(PROBLEM_NAMES))


if __name__ == "__main__":
    main()
