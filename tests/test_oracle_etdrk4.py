"""ETDRK4 in the oracle, checked without the reference (no reference test
exercises it): the contour-integral coefficients against the φ-function
closed forms evaluated in 100-digit arithmetic, and the stepper's order of
convergence on an advection-diffusion solve (4 for ETDRK4 and for RK4, the
two agreeing as dt shrinks).  The GPU path matches the oracle's ETDRK4 to
1e-12 (FP64), so these bounds carry over to it."""
import math

import numpy as np
import pytest

Z = [0.0, -1e-8, -1e-4, -0.01, -0.3, -0.95, -1.0, -1.05, -2.5, -10.0, -100.0, -1e3, -1e4]
# 32 points on a unit circle about z: relative error <= 1e-12 over z in
# [-1e4, 0]; the worst (5e-13) is at |z| ~ 1, where the circle passes close
# to the origin and the closed forms cancel there.
COEF_RTOL = 1e-12


def _exact(z, dt):
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 100
    if z == 0.0:  # limits of the closed forms
        return (1.0, 1.0, dt / 2, dt / 6, dt / 6, dt / 6)
    zz = mp.mpf(z)
    ez = mp.e ** zz
    zeta = (mp.e ** (zz / 2) - 1) / zz
    alpha = (-4 - zz + ez * (4 - 3 * zz + zz ** 2)) / zz ** 3
    beta = (2 + zz + ez * (zz - 2)) / zz ** 3
    gamma = (-4 - 3 * zz - zz ** 2 + ez * (4 - zz)) / zz ** 3
    return (float(ez), float(mp.e ** (zz / 2)), dt * float(zeta), dt * float(alpha), dt * float(beta),
            dt * float(gamma))


@pytest.mark.parametrize("dt", [0.002, 0.05])
def test_etd_coefficients_match_closed_forms(oracle, dt):
    L = np.array(Z) / dt
    got = oracle.etdrk4_coefficients(dt, L)
    for i, z in enumerate(Z):
        want = _exact(z, dt)
        for name, g, w in zip(("E", "E2", "zeta", "alpha", "beta", "gamma"), (a[i] for a in got), want):
            assert abs(g - w) <= COEF_RTOL * abs(w), (name, z, g, w)


def _solve(oracle, stepper, dt, T=0.32, n=32):
    u = lambda x, y: np.cos(x) * np.sin(y) + 0.3
    v = lambda x, y: -np.sin(x) * np.cos(y)
    p = oracle.Problem(oracle.TwoDAdvectingFlow(u=u, v=v), nx=n, kappa=0.05, eta=0.05, dt=dt, stepper=stepper)
    x = -np.pi + 2 * np.pi / n * np.arange(n)
    Y, X = np.meshgrid(x, x, indexing="ij")
    oracle.set_c(p, np.exp(-(X ** 2 + Y ** 2) / 0.8) + 0.2 * np.cos(X + 2 * Y))
    oracle.stepforward(p, int(round(T / dt)))
    oracle.updatevars(p)
    return p.vars.c.copy()


@pytest.mark.parametrize("stepper", ["ETDRK4", "RK4"])
def test_fourth_order_convergence(oracle, stepper):
    ref = _solve(oracle, stepper, 0.32 / 512)
    errs = [np.linalg.norm(_solve(oracle, stepper, 0.32 / m) - ref) for m in (16, 32, 64)]
    orders = [math.log2(errs[i] / errs[i + 1]) for i in range(2)]
    assert all(3.9 <= q <= 4.1 for q in orders), (errs, orders)  # measured 4.00-4.01


def test_etdrk4_and_rk4_agree_as_dt_shrinks(oracle):
    d = [np.linalg.norm(_solve(oracle, "ETDRK4", 0.32 / m) - _solve(oracle, "RK4", 0.32 / m)) for m in (32, 128)]
    assert d[1] < d[0] / 100 and d[1] < 1e-8
