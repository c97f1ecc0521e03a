"""Exact solution of the one-dimensional Riemann problem for the Euler
equations of an ideal gas, for the physics checks of the tests.

The method is the textbook one (E. F. Toro, "Riemann Solvers and Numerical
Methods for Fluid Dynamics", 3rd ed., Springer 2009, chapter 4): the star
pressure is the root of f_L(p) + f_R(p) + (u_R - u_L) = 0, with f_K the
shock (Rankine-Hugoniot) or rarefaction (isentropic) branch of each side,
found by Newton iteration from the primitive-variable guess; the solution is
then sampled along x/t across the left wave, the contact and the right wave.
"""
import math

import numpy as np


def _f(p, rho, pk, c, g):
    """Pressure function of one side and its derivative."""
    if p > pk:  # shock
        a = 2.0 / ((g + 1.0) * rho)
        b = (g - 1.0) / (g + 1.0) * pk
        q = math.sqrt(a / (p + b))
        return (p - pk) * q, q * (1.0 - 0.5 * (p - pk) / (b + p))
    r = p / pk  # rarefaction
    return (2.0 * c / (g - 1.0)) * (r ** ((g - 1.0) / (2.0 * g)) - 1.0), r ** (-(g + 1.0) / (2.0 * g)) / (rho * c)


def star_state(left, right, g):
    """(p*, u*) of the Riemann problem left = (rho, u, p), right = (rho, u, p)."""
    rl, ul, pl = left
    rr, ur, pr = right
    cl, cr = math.sqrt(g * pl / rl), math.sqrt(g * pr / rr)
    if 2.0 * (cl + cr) / (g - 1.0) <= ur - ul:
        raise ValueError("the data generate vacuum")
    p = max(1e-12, 0.5 * (pl + pr) - 0.125 * (ur - ul) * (rl + rr) * (cl + cr))
    for _ in range(100):
        fl, dl = _f(p, rl, pl, cl, g)
        fr, dr = _f(p, rr, pr, cr, g)
        p_new = max(1e-12, p - (fl + fr + ur - ul) / (dl + dr))
        done = abs(p_new - p) <= 1e-14 * 0.5 * (p_new + p)
        p = p_new
        if done:
            break
    fl, _ = _f(p, rl, pl, cl, g)
    fr, _ = _f(p, rr, pr, cr, g)
    return p, 0.5 * (ul + ur) + 0.5 * (fr - fl)


def sample(left, right, g, s):
    """(rho, u, p) at the similarity coordinate s = (x - x0) / t."""
    ps, us = star_state(left, right, g)
    if s <= us:
        rk, uk, pk, sgn = left[0], left[1], left[2], 1.0
    else:
        rk, uk, pk, sgn = right[0], right[1], right[2], -1.0
    c = math.sqrt(g * pk / rk)
    # write the right side as a mirrored left side: u -> -u, s -> -s
    uk_, us_, s_ = sgn * uk, sgn * us, sgn * s
    if ps > pk:  # shock
        sh = uk_ - c * math.sqrt((g + 1.0) / (2.0 * g) * ps / pk + (g - 1.0) / (2.0 * g))
        if s_ <= sh:
            return rk, uk, pk
        g6 = (g - 1.0) / (g + 1.0)
        return rk * (ps / pk + g6) / (g6 * ps / pk + 1.0), us, ps
    head = uk_ - c  # rarefaction
    if s_ <= head:
        return rk, uk, pk
    cs = c * (ps / pk) ** ((g - 1.0) / (2.0 * g))
    if s_ > us_ - cs:
        return rk * (ps / pk) ** (1.0 / g), us, ps
    u_ = 2.0 / (g + 1.0) * (c + 0.5 * (g - 1.0) * uk_ + s_)
    cf = 2.0 / (g + 1.0) * (c + 0.5 * (g - 1.0) * (uk_ - s_))
    return rk * (cf / c) ** (2.0 / (g - 1.0)), sgn * u_, pk * (cf / c) ** (2.0 * g / (g - 1.0))


def profile(left, right, g, x, x0, t):
    """rho, u, p arrays at positions x and time t > 0."""
    out = np.array([sample(left, right, g, (xi - x0) / t) for xi in x])
    return out[:, 0], out[:, 1], out[:, 2]
