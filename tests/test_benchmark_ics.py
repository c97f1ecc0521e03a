"""The three FP64 benchmark set-ups' initial conditions against their stated
definitions, on the oracle (the GPU's are compared with the oracle bitwise
in the GPU tests):
* Sedov: rho = 1, u = v = 0, p = 1e-5, and p = (gamma - 1) E0 / (pi r0^2)
  with E0 = 1 in the cells whose centre lies within r0 = 0.02 of (0.5, 0.5);
* Kelvin-Helmholtz: rho = 2, u = +0.5 for |y - 0.5| < 0.25, else rho = 1,
  u = -0.5; p = 2.5; v = 0.01 sin(4 pi x); seeded uniform noise of amplitude
  1e-3 on u and v;
* Rayleigh-Taylor: rho = 2 above y = 0.75, 1 below; hydrostatic p under
  g = -0.1 with p = 2.5 at the interface; v = 0.01 (1 + cos 4 pi x)
  (1 + cos 3 pi (y - 0.75)) / 4."""
import numpy as np

from fv2d_testlib import Oracle, reference_params


def centres(p):
    dx, dy = (p.xmax - p.xmin) / p.Nx, (p.ymax - p.ymin) / p.Ny
    x = p.xmin + (np.arange(p.Nx) + 0.5) * dx
    y = p.ymin + (np.arange(p.Ny) + 0.5) * dy
    return np.meshgrid(x, y)


def test_sedov_initial_condition():
    p = reference_params(Nx=512, Ny=512, gamma0=1.4, reconstruction=2, riemann_solver=1, boundary_x=1, boundary_y=1)
    o = Oracle(p)
    o.init_problem("sedov")
    q = o.get_prim()
    X, Y = centres(p)
    inside = np.hypot(X - 0.5, Y - 0.5) <= 0.02
    assert 20 < inside.sum() < 400
    assert np.all(q[..., 0] == 1.0) and np.all(q[..., 1] == 0.0) and np.all(q[..., 2] == 0.0)
    p_in = (p.gamma0 - 1.0) * 1.0 / (np.pi * 0.02 ** 2)
    assert np.allclose(q[..., 3][inside], p_in, rtol=1e-15) and np.all(q[..., 3][~inside] == 1e-5)


def test_kelvin_helmholtz_initial_condition():
    p = reference_params(Nx=512, Ny=512, gamma0=1.4, reconstruction=2, riemann_solver=1, boundary_x=2, boundary_y=2)
    o = Oracle(p)
    o.init_problem("kh_step")
    q = o.get_prim()
    X, Y = centres(p)
    band = np.abs(Y - 0.5) < 0.25
    assert np.all(q[..., 0][band] == 2.0) and np.all(q[..., 0][~band] == 1.0) and np.all(q[..., 3] == 2.5)
    du = q[..., 1] - np.where(band, 0.5, -0.5)
    dv = q[..., 2] - 0.01 * np.sin(4 * np.pi * X)
    for d in (du, dv):
        assert np.abs(d).max() <= 1e-3 + 1e-15
        assert abs(d.std() - 1e-3 / np.sqrt(3)) < 2e-5 and abs(d.mean()) < 2e-5   # uniform on [-1e-3, 1e-3]
    assert abs(np.corrcoef(du.ravel(), dv.ravel())[0, 1]) < 0.01                   # independent streams


def test_rayleigh_taylor_initial_condition():
    p = reference_params(Nx=128, Ny=384, xmax=0.5, ymax=1.5, gamma0=1.4, reconstruction=2, riemann_solver=0,
                         boundary_x=2, boundary_y=1, gravity_mode=1, gy=-0.1)
    o = Oracle(p)
    o.init_problem("rt_hydrostatic")
    q = o.get_prim()
    X, Y = centres(p)
    rho = np.where(Y > 0.75, 2.0, 1.0)
    assert np.all(q[..., 0] == rho) and np.all(q[..., 1] == 0.0)
    assert np.allclose(q[..., 3], 2.5 + rho * p.gy * (Y - 0.75), rtol=1e-14, atol=1e-15)
    v = 0.01 * (1 + np.cos(4 * np.pi * X)) * (1 + np.cos(3 * np.pi * (Y - 0.75))) / 4
    assert np.allclose(q[..., 2], v, rtol=1e-13, atol=1e-17)
    assert abs(p.gy - (-0.1)) < 1e-8   # -0.1 as the reference reads it (float-rounded)
