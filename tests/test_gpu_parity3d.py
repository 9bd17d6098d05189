"""3D GPU parity through the C ABI (src/traceradvectiondiffusion.jl:771-786)."""
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
FP32_TOL = 1e-5
GOLD = Path(__file__).resolve().parent / "golden"


def abc(A=1.0, B=np.sqrt(2 / 3), C=np.sqrt(1 / 3)):
    return (lambda x, y, z: A * np.sin(z) + C * np.cos(y), lambda x, y, z: B * np.sin(x) + A * np.cos(z),
            lambda x, y, z: C * np.sin(y) + B * np.cos(x))


def gauss3(x, y, z, s=0.3, c=(0.0, 0.0, 0.0)):
    return np.exp(-((x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2) / (2 * s ** 2))


def pair(gpu, oracle, n, ny=None, nz=None, stepper="RK4", T=np.float64, dt=0.002, κ=5e-4, η=4e-4, ι=3e-4,
         κh=0.0, nκh=0, L=(2 * np.pi, 2 * np.pi, 2 * np.pi)):
    ny, nz = ny or n, nz or n
    u, v, w = abc()
    kw = dict(nx=n, ny=ny, nz=nz, Lx=L[0], Ly=L[1], Lz=L[2], dt=dt, stepper=stepper)
    p = gpu.Problem(gpu.GPU(), gpu.ThreeDAdvectingFlow(u=u, v=v, w=w), κ=κ, η=η, ι=ι, κh=κh, nκh=nκh, T=T, **kw)
    r = oracle.Problem(oracle.ThreeDAdvectingFlow(u=u, v=v, w=w), kappa=κ, eta=η, iota=ι, kappah=κh, nkappah=nκh, **kw)
    return p, r


def advance(gpu, oracle, p, r, c0, nsteps):
    gpu.set_c(p, c0); oracle.set_c(r, c0)
    gpu.stepforward(p, nsteps); oracle.stepforward(r, nsteps)
    gpu.updatevars(p); oracle.updatevars(r)
    return oracle.rel_l2(p.vars.c, r.vars.c)


@pytest.mark.parametrize("n,ny,nz", [(16, 16, 16), (32, 32, 32), (64, 64, 64), (32, 64, 16), (64, 16, 32)])
@pytest.mark.parametrize("stepper", ["RK4", "ETDRK4"])
def test_3d_fp64(gpu, oracle, n, ny, nz, stepper):
    p, r = pair(gpu, oracle, n, ny, nz, stepper=stepper, L=(2 * np.pi, 5.0, 7.0))
    x, y, z = gpu.gridpoints(p.grid)
    assert advance(gpu, oracle, p, r, gauss3(x, y, z, 0.5, (0.2, -0.3, 0.1)), 5) <= FP64_TOL


def test_3d_hyperdiffusion_fp64(gpu, oracle):
    p, r = pair(gpu, oracle, 32, stepper="ETDRK4", κh=1e-6, nκh=2)
    x, y, z = gpu.gridpoints(p.grid)
    assert advance(gpu, oracle, p, r, gauss3(x, y, z), 6) <= FP64_TOL


@pytest.mark.parametrize("stepper", ["RK4", "ETDRK4"])
def test_3d_fp32(gpu, oracle, stepper):
    p, r = pair(gpu, oracle, 64, stepper=stepper, T=np.float32, dt=0.005)
    x, y, z = gpu.gridpoints(p.grid)
    assert advance(gpu, oracle, p, r, gauss3(x, y, z), 10) <= FP32_TOL


def test_3d_calcN(gpu, oracle):
    p, r = pair(gpu, oracle, 32, 16, 64)
    x, y, z = gpu.gridpoints(p.grid)
    sol = r.grid.rfft(gauss3(x, y, z, 0.6) + 0.2 * np.sin(x) * np.cos(2 * y) * np.sin(3 * z))
    Ng = p.calcN(sol)
    Nr = np.empty_like(sol)
    oracle.calcN(Nr, sol, 0.0, r.clock, r.params, r.grid)
    assert oracle.rel_l2(Ng, Nr) <= 1e-13


@pytest.mark.parametrize("n,T,tol", [(16, np.float64, 1e-15), (128, np.float64, 1e-15), (64, np.float32, 5e-7)])
def test_3d_set_c_roundtrip(gpu, oracle, n, T, tol):
    p, r = pair(gpu, oracle, n, T=T)
    c = np.random.default_rng(n).standard_normal(p.grid.shape)
    gpu.set_c(p, c)
    assert oracle.rel_l2(p.vars.c, c) <= tol
    assert oracle.rel_l2(p.sol, r.grid.rfft(c)) <= tol


def test_3d_256_one_step(gpu, oracle):
    """Config-3 size (256³, ETDRK4, ABC flow, κ=5e-4): one step against the oracle."""
    p, r = pair(gpu, oracle, 256, stepper="ETDRK4", dt=0.005, κ=5e-4, η=5e-4, ι=5e-4)
    x, y, z = gpu.gridpoints(p.grid)
    assert advance(gpu, oracle, p, r, gauss3(x, y, z), 1) <= FP64_TOL


def test_3d_batch_equals_separate(gpu, oracle):
    u, v, w = abc()
    kw = dict(nx=32, κ=5e-4, dt=0.005, stepper="ETDRK4")
    p = gpu.Problem(gpu.GPU(), gpu.ThreeDAdvectingFlow(u=u, v=v, w=w), batch=2, **kw)
    x, y, z = gpu.gridpoints(p.grid)
    cs = np.stack([gauss3(x, y, z, 0.4, (0.1 * b, 0, -0.2 * b)) for b in range(2)])
    gpu.set_c(p, cs); gpu.stepforward(p, 4); gpu.updatevars(p)
    for b in range(2):
        q = gpu.Problem(gpu.GPU(), gpu.ThreeDAdvectingFlow(u=u, v=v, w=w), **kw)
        gpu.set_c(q, cs[b]); gpu.stepforward(q, 4); gpu.updatevars(q)
        assert np.array_equal(q.vars.c, p.vars.c[b])


def test_golden_abc32(gpu, oracle):
    g = np.load(GOLD / "abc32_etdrk4.npz")
    u, v, w = abc()
    for T, tol in ((np.float64, 1e-12), (np.float32, 1e-5)):
        p = gpu.Problem(gpu.GPU(), gpu.ThreeDAdvectingFlow(u=u, v=v, w=w), nx=32, κ=5e-4, dt=0.005,
                        stepper="ETDRK4", T=T)
        gpu.set_c(p, g["c0"]); gpu.stepforward(p, 100); gpu.updatevars(p)
        assert oracle.rel_l2(p.vars.c, g["c100"]) <= tol, T
