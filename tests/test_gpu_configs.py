"""The benchmark configurations at their configured grid sizes, against the
FP64 CPU oracle (``oracle/ptf_oracle.py``).

* 2D cellular flow ψ = cos(4x) cos(4y), κ = η = 1e-4, κh = 1e-12 on ∇⁴
  (nκh = 2), Gaussian σ = 0.2 at (π/2, π/2), ETDRK4, at 4096²: 20 steps at
  full size.  The configured dt = 2e-3 gives an advective CFL number
  u_max·k_max·dt = 4·2048·2e-3 ≈ 16 at 4096², far beyond the ETDRK4
  stability limit (≈2.8), where every solution diverges; dt = 1e-4 (CFL
  0.82) is used.  The cost of a step does not depend on dt.
* 3D ABC flow (A = 1, B = √(2/3), C = √(1/3)), κ = η = ι = 5e-4, Gaussian
  σ = 0.3 at the centre, ETDRK4, dt = 0.005, at 256³: FP64 against the
  oracle over 20 steps at full size, and FP32 against the FP64 GPU path
  over the configured 500 steps.

Tolerances (relative L2 of the physical field): FP64 1e-10 (the drop-in
target against the reference); FP32 1e-5.  Mass drift sum(c_end)/sum(c0) - 1
is compared with the oracle's own drift (the advective form conserves the
k = 0 mode only up to aliasing): FP64 to 1e-12, FP32 (FP64 k = 0 mode) to
1e-9 over 20 steps and 1e-7 over the 500 steps of 256^3.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10
FP32_TOL = 1e-5


def _cellular4():
    return (lambda x, y: 4 * np.cos(4 * x) * np.sin(4 * y), lambda x, y: -4 * np.sin(4 * x) * np.cos(4 * y))


def _drift(c, m0):
    return float(np.sum(c)) / m0 - 1.0


def test_config_2d_4096_etdrk4_vs_oracle(gpu, oracle):
    n, dt, steps = 4096, 1e-4, 20
    u, v = _cellular4()
    kw = dict(nx=n, Lx=2 * np.pi, dt=dt, stepper="ETDRK4")
    r = oracle.Problem(oracle.TwoDAdvectingFlow(u=u, v=v), kappa=1e-4, eta=1e-4, kappah=1e-12, nkappah=2, **kw)
    x = r.grid.x
    X, Y = np.meshgrid(x, x)
    c0 = np.exp(-((X - np.pi / 2) ** 2 + (Y - np.pi / 2) ** 2) / (2 * 0.2 ** 2))
    m0 = float(c0.sum())
    oracle.set_c(r, c0)
    oracle.stepforward(r, steps)
    oracle.updatevars(r)
    ref = r.vars.c
    for T, tol, dtol in ((np.float64, FP64_TOL, 1e-12), (np.float32, FP32_TOL, 1e-9)):
        p = gpu.Problem(gpu.GPU(), gpu.TwoDAdvectingFlow(u=u, v=v), κ=1e-4, η=1e-4, κh=1e-12, nκh=2, T=T, **kw)
        gpu.set_c(p, c0)
        gpu.stepforward(p, steps)
        gpu.updatevars(p)
        assert oracle.rel_l2(p.vars.c, ref) <= tol
        assert abs(_drift(p.vars.c, m0) - _drift(ref, m0)) <= dtol
        del p


def _abc():
    A, B, C = 1.0, np.sqrt(2 / 3), np.sqrt(1 / 3)
    return (lambda x, y, z: A * np.sin(z) + C * np.cos(y), lambda x, y, z: B * np.sin(x) + A * np.cos(z),
            lambda x, y, z: C * np.sin(y) + B * np.cos(x))


def _abc_ic(n):
    x = -np.pi + 2 * np.pi / n * np.arange(n)
    Z, Y, X = np.meshgrid(x, x, x, indexing="ij")
    return np.exp(-(X ** 2 + Y ** 2 + Z ** 2) / (2 * 0.3 ** 2))


def test_config_3d_abc_256_fp64_vs_oracle(gpu, oracle):
    n, dt, steps = 256, 0.005, 20
    u, v, w = _abc()
    r = oracle.Problem(oracle.ThreeDAdvectingFlow(u=u, v=v, w=w), nx=n, kappa=5e-4, dt=dt, stepper="ETDRK4")
    c0 = _abc_ic(n)
    m0 = float(c0.sum())
    oracle.set_c(r, c0)
    oracle.stepforward(r, steps)
    oracle.updatevars(r)
    p = gpu.Problem(gpu.GPU(), gpu.ThreeDAdvectingFlow(u=u, v=v, w=w), nx=n, κ=5e-4, dt=dt, stepper="ETDRK4",
                    T=np.float64)
    gpu.set_c(p, c0)
    gpu.stepforward(p, steps)
    gpu.updatevars(p)
    assert oracle.rel_l2(p.vars.c, r.vars.c) <= FP64_TOL
    assert abs(_drift(p.vars.c, m0) - _drift(r.vars.c, m0)) <= 1e-12


def test_config_3d_abc_256_fp32_500_steps(gpu, oracle):
    """The configured length, FP32 against the FP64 GPU path (the oracle at
    256³ for 500 steps takes tens of minutes of CPU; the FP64 path is pinned
    to it over 20 steps above)."""
    n, dt, steps = 256, 0.005, 500
    u, v, w = _abc()
    c0 = _abc_ic(n)
    m0 = float(c0.sum())
    out = {}
    for T in (np.float64, np.float32):
        p = gpu.Problem(gpu.GPU(), gpu.ThreeDAdvectingFlow(u=u, v=v, w=w), nx=n, κ=5e-4, dt=dt, stepper="ETDRK4",
                        T=T)
        gpu.set_c(p, c0)
        gpu.stepforward(p, steps)
        gpu.updatevars(p)
        out[T] = p.vars.c.copy()
        del p
    assert oracle.rel_l2(out[np.float32], out[np.float64]) <= FP32_TOL
    # N(0,0,0) is a compensated FP64 sum of FP32 transform outputs; their
    # rounding random-walks over 2000 right-hand sides of 256^3 points
    assert abs(_drift(out[np.float32], m0) - _drift(out[np.float64], m0)) <= 1e-7
