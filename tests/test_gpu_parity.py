"""GPU parity: the CUDA path (through the C ABI) against the FP64 CPU oracle.

Tolerances (relative L2 of the physical field):
  FP64: 1e-12 after a few steps (the reference target is <= 1e-10)
  FP32: 1e-5 (FP32 bulk transforms, FP64 tables)
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
FP32_TOL = 1e-5


def cellular(k=1.0, U=1.0):
    return (lambda x, y: U * k * np.cos(k * x) * np.sin(k * y), lambda x, y: -U * k * np.sin(k * x) * np.cos(k * y))


def gauss(x, y, x0=np.pi / 2, y0=np.pi / 2, s=0.2):
    return np.exp(-((x - x0) ** 2 + (y - y0) ** 2) / (2 * s ** 2))


def pair(gpu, oracle, n, ny=None, stepper="RK4", T=np.float64, dt=0.002, κ=0.002, η=0.001, κh=0.0, nκh=0,
         k=1.0, Lx=2 * np.pi, Ly=None, batch=1):
    ny = ny or n
    Ly = Ly or Lx
    u, v = cellular(k)
    kw = dict(nx=n, ny=ny, Lx=Lx, Ly=Ly, dt=dt, stepper=stepper)
    p = gpu.Problem(gpu.GPU(), gpu.TwoDAdvectingFlow(u=u, v=v), κ=κ, η=η, κh=κh, nκh=nκh, T=T, batch=batch, **kw)
    r = oracle.Problem(oracle.TwoDAdvectingFlow(u=u, v=v), kappa=κ, eta=η, kappah=κh, nkappah=nκh, **kw)
    return p, r


def advance(gpu, oracle, p, r, c0, nsteps):
    gpu.set_c(p, c0)
    oracle.set_c(r, c0)
    gpu.stepforward(p, nsteps)
    oracle.stepforward(r, nsteps)
    gpu.updatevars(p)
    oracle.updatevars(r)
    return oracle.rel_l2(p.vars.c, r.vars.c)


@pytest.mark.parametrize("n", [16, 32, 64, 128, 256, 512, 1024])
def test_rk4_fp64_square(gpu, oracle, n):
    p, r = pair(gpu, oracle, n, dt=min(0.002, 2.0 / (0.002 * (n / 2) ** 2) / 4))
    x, y = gpu.gridpoints(p.grid)
    assert advance(gpu, oracle, p, r, gauss(x, y), 6) <= FP64_TOL


@pytest.mark.parametrize("n,ny,Lx,Ly", [(128, 64, 2 * np.pi, 2 * np.pi), (64, 256, 2 * np.pi, 4.0),
                                        (32, 512, 3.0, 2 * np.pi), (512, 16, 2 * np.pi, 2 * np.pi)])
def test_rk4_fp64_rectangular(gpu, oracle, n, ny, Lx, Ly):
    p, r = pair(gpu, oracle, n, ny=ny, Lx=Lx, Ly=Ly, dt=0.001)
    x, y = gpu.gridpoints(p.grid)
    assert advance(gpu, oracle, p, r, gauss(x, y, 0.3, -0.2), 5) <= FP64_TOL


@pytest.mark.parametrize("n", [64, 256, 1024])
def test_etdrk4_fp64_hyperdiffusion(gpu, oracle, n):
    p, r = pair(gpu, oracle, n, stepper="ETDRK4", κ=1e-4, η=1e-4, κh=1e-9, nκh=2, k=4.0, dt=0.0005)
    x, y = gpu.gridpoints(p.grid)
    assert advance(gpu, oracle, p, r, gauss(x, y), 6) <= FP64_TOL


@pytest.mark.parametrize("n", [2048, 4096])
def test_fp64_large_one_step(gpu, oracle, n):
    p, r = pair(gpu, oracle, n, stepper="ETDRK4", κ=1e-4, η=1e-4, κh=1e-12, nκh=2, k=4.0, dt=0.0002)
    x, y = gpu.gridpoints(p.grid)
    assert advance(gpu, oracle, p, r, gauss(x, y), 1) <= FP64_TOL


@pytest.mark.parametrize("n,stepper", [(64, "RK4"), (256, "RK4"), (1024, "ETDRK4"), (256, "ETDRK4")])
def test_fp32(gpu, oracle, n, stepper):
    p, r = pair(gpu, oracle, n, stepper=stepper, T=np.float32, dt=0.0005, κ=1e-3, η=1e-3)
    x, y = gpu.gridpoints(p.grid)
    assert advance(gpu, oracle, p, r, gauss(x, y), 10) <= FP32_TOL


@pytest.mark.parametrize("n,T,tol", [(64, np.float64, 1e-13), (512, np.float64, 1e-13), (256, np.float32, 2e-6)])
def test_calcN_plugin(gpu, oracle, n, T, tol):
    """ptf_calcN == calcN! (src/traceradvectiondiffusion.jl:756-769) on the same spectral input."""
    p, r = pair(gpu, oracle, n, T=T)
    x, y = gpu.gridpoints(p.grid)
    sol = r.grid.rfft(gauss(x, y) + 0.3 * np.sin(2 * x) * np.cos(3 * y))
    Ng = p.calcN(sol)
    Nr = np.empty_like(sol)
    oracle.calcN(Nr, sol, 0.0, r.clock, r.params, r.grid)
    assert oracle.rel_l2(Ng, Nr) <= tol


@pytest.mark.parametrize("n,T,tol", [(16, np.float64, 1e-15), (1024, np.float64, 1e-15), (4096, np.float64, 1e-15),
                                     (512, np.float32, 5e-7)])
def test_set_c_roundtrip_and_sol(gpu, oracle, n, T, tol):
    p, r = pair(gpu, oracle, n, T=T)
    rng = np.random.default_rng(n)
    c = rng.standard_normal(p.grid.shape)
    gpu.set_c(p, c)
    assert oracle.rel_l2(p.vars.c, c) <= tol
    assert oracle.rel_l2(p.sol, r.grid.rfft(c)) <= tol


def test_set_sol_get_sol(gpu, oracle):
    p, r = pair(gpu, oracle, 64)
    x, y = gpu.gridpoints(p.grid)
    sol = r.grid.rfft(gauss(x, y))
    p.sol = sol
    assert np.array_equal(p.sol, sol)
    gpu.updatevars(p)
    assert oracle.rel_l2(p.vars.c, gauss(x, y)) <= 1e-15


def test_batch_equals_separate_solves(gpu, oracle):
    """A batch of independent solves gives bit-identical results to solving each alone."""
    n, B = 128, 3
    p, _ = pair(gpu, oracle, n, batch=B)
    x, y = gpu.gridpoints(p.grid)
    cs = np.stack([gauss(x, y, 0.5 * b, -0.4 * b, 0.2 + 0.05 * b) for b in range(B)])
    gpu.set_c(p, cs)
    gpu.stepforward(p, 7)
    gpu.updatevars(p)
    for b in range(B):
        q, _ = pair(gpu, oracle, n)
        gpu.set_c(q, cs[b])
        gpu.stepforward(q, 7)
        gpu.updatevars(q)
        assert np.array_equal(q.vars.c, p.vars.c[b])


def test_time_varying_flow_clock_t(gpu, oracle):
    """Time-varying flow evaluated at clock.t for all four stages (:708-723)."""
    n, dt = 64, 0.004
    u = lambda x, y, t: np.cos(x + 0.3 * np.sin(t)) * np.sin(y)
    v = lambda x, y, t: -np.sin(x + 0.3 * np.sin(t)) * np.cos(y)
    p = gpu.Problem(gpu.GPU(), gpu.TwoDAdvectingFlow(u=u, v=v, steadyflow=False), nx=n, κ=1e-3, dt=dt)
    r = oracle.Problem(oracle.TwoDAdvectingFlow(u=u, v=v, steadyflow=False), nx=n, kappa=1e-3, dt=dt)
    x, y = gpu.gridpoints(p.grid)
    assert advance(gpu, oracle, p, r, gauss(x, y), 8) <= FP64_TOL
    assert p.clock.step == 8 and abs(p.clock.t - 8 * dt) < 1e-15


def test_step_split_equals_single_call(gpu, oracle):
    p, _ = pair(gpu, oracle, 64)
    q, _ = pair(gpu, oracle, 64)
    x, y = gpu.gridpoints(p.grid)
    gpu.set_c(p, gauss(x, y)); gpu.set_c(q, gauss(x, y))
    gpu.stepforward(p, 6)
    for _ in range(3):
        gpu.stepforward(q, 2)
    gpu.updatevars(p); gpu.updatevars(q)
    assert np.array_equal(p.vars.c, q.vars.c)


def test_errors_are_raised_not_faults(gpu):
    from ptf_gb300._lib import PtfError
    p = gpu.Problem(gpu.GPU(), gpu.TwoDAdvectingFlow(), nx=32)
    with pytest.raises(PtfError):
        gpu.stepforward(p, 1)  # no initial condition yet
    with pytest.raises(ValueError):
        gpu.stepforward(p, -1)


def test_golden_cellular128_rk4_2000_steps(gpu, oracle):
    """The 128² cellular-flow workload (RK4, dt=0.01, 2000 steps, FP64) vs the
    golden fixture: the reference target is <= 1e-10."""
    from pathlib import Path
    g = np.load(Path(__file__).resolve().parent / "golden" / "cellular128_rk4.npz")
    u, v = cellular()
    p = gpu.Problem(gpu.GPU(), gpu.TwoDAdvectingFlow(u=u, v=v), nx=128, κ=0.002, η=0.0, dt=0.01)
    gpu.set_c(p, g["c0"])
    gpu.stepforward(p, 100); gpu.updatevars(p)
    assert oracle.rel_l2(p.vars.c, g["c100"]) <= 1e-12
    gpu.stepforward(p, 1900); gpu.updatevars(p)
    assert oracle.rel_l2(p.vars.c, g["c2000"]) <= 1e-10
    assert p.clock.step == 2000


def test_golden_etdrk4_fp64_fp32(gpu, oracle):
    from pathlib import Path
    g = np.load(Path(__file__).resolve().parent / "golden" / "cellular128_etdrk4.npz")
    u, v = cellular(4.0)
    for T, tol in ((np.float64, 1e-10), (np.float32, 1e-5)):
        p = gpu.Problem(gpu.GPU(), gpu.TwoDAdvectingFlow(u=u, v=v), nx=128, κ=1e-4, η=1e-4, κh=1e-12, nκh=2,
                        dt=0.002, stepper="ETDRK4", T=T)
        x, y = gpu.gridpoints(p.grid)
        gpu.set_c(p, gauss(x, y))
        gpu.stepforward(p, 50); gpu.updatevars(p)
        assert oracle.rel_l2(p.vars.c, g["c50"]) <= tol, T


@pytest.mark.parametrize("T,tol", [(np.float64, 1e-12), (np.float32, 1e-5)])
def test_analytic_cellular_flow_on_device(gpu, oracle, T, tol):
    """ptf_set_flow_analytic: the time-dependent cellular flow evaluated on the
    device at clock.t before every step equals the same flow given as a Python
    function (evaluated on the host at clock.t) -- and the oracle."""
    U, eps, om, Kx, Ky = 0.8, 0.4, 3.0, 2, 1
    k, l = float(Kx), float(Ky)
    u = lambda x, y, t: U * l * np.cos(k * x + eps * np.sin(om * t)) * np.sin(l * y)  # noqa: E731
    v = lambda x, y, t: -U * k * np.sin(k * x + eps * np.sin(om * t)) * np.cos(l * y)  # noqa: E731
    kw = dict(nx=128, dt=0.004, stepper="RK4")
    p = gpu.Problem(gpu.GPU(), gpu.TwoDAdvectingFlow(), κ=1e-3, T=T, **kw)
    p.set_flow_analytic("cellular", U=U, eps=eps, omega=om, Kx=Kx, Ky=Ky)
    q = gpu.Problem(gpu.GPU(), gpu.TwoDAdvectingFlow(u=u, v=v, steadyflow=False), κ=1e-3, T=T, **kw)
    r = oracle.Problem(oracle.TwoDAdvectingFlow(u=u, v=v, steadyflow=False), kappa=1e-3, **kw)
    x, y = gpu.gridpoints(p.grid)
    c0 = gauss(x, y, 0.2, -0.5, 0.4)
    for prob in (p, q):
        gpu.set_c(prob, c0)
        gpu.stepforward(prob, 25)
        gpu.updatevars(prob)
    oracle.set_c(r, c0)
    oracle.stepforward(r, 25)
    oracle.updatevars(r)
    assert oracle.rel_l2(p.vars.c, q.vars.c) <= (1e-13 if T is np.float64 else 1e-6)
    assert oracle.rel_l2(p.vars.c, r.vars.c) <= tol
    # calcN! at clock.t with the device-evaluated flow
    N = p.calcN(p.sol)
    Nr = np.zeros_like(r.sol)
    oracle.calcN(Nr, r.sol, r.clock.t, r.clock, r.params, r.grid)
    if T is np.float64:
        assert oracle.rel_l2(N, Nr) <= 1e-12


def test_analytic_abc_flow_on_device(gpu, oracle):
    A, B, C = 1.0, np.sqrt(2 / 3), np.sqrt(1 / 3)
    fu = lambda x, y, z: A * np.sin(z) + C * np.cos(y)  # noqa: E731
    fv = lambda x, y, z: B * np.sin(x) + A * np.cos(z)  # noqa: E731
    fw = lambda x, y, z: C * np.sin(y) + B * np.cos(x)  # noqa: E731
    kw = dict(nx=32, dt=0.005, stepper="ETDRK4")
    p = gpu.Problem(gpu.GPU(), gpu.ThreeDAdvectingFlow(), κ=5e-4, **kw)
    p.set_flow_analytic("abc", A=A, B=B, C=C)
    r = oracle.Problem(oracle.ThreeDAdvectingFlow(u=fu, v=fv, w=fw), kappa=5e-4, **kw)
    x, y, z = gpu.gridpoints(p.grid)
    c0 = np.exp(-(x ** 2 + y ** 2 + z ** 2) / (2 * 0.3 ** 2))
    gpu.set_c(p, c0)
    oracle.set_c(r, c0)
    gpu.stepforward(p, 10)
    oracle.stepforward(r, 10)
    gpu.updatevars(p)
    oracle.updatevars(r)
    assert oracle.rel_l2(p.vars.c, r.vars.c) <= 1e-12
    with pytest.raises(Exception):
        p.set_flow_analytic("cellular")  # the cellular flow is 2D
