"""1D path (src/traceradvectiondiffusion.jl:143-163, :744-754): the GPU
through the C ABI against the FP64 oracle.  Solves are stepped in pairs; odd
batches carry one zero solve on the device, so batch sizes 1 and 3 are
covered.

Tolerances (relative L2): FP64 1e-12, FP32 1e-5; calcN 1e-13 (FP64).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def flow1(k=2.0):
    return lambda x: 0.7 + 0.5 * np.sin(k * x)


def ic1(x, x0=0.4, s=0.25):
    return np.exp(-((x - x0) ** 2) / (2 * s ** 2)) + 0.2 * np.cos(3 * x)


def pair1(gpu, oracle, n, stepper="RK4", T=np.float64, dt=0.002, κ=0.003, κh=0.0, nκh=0, Lx=2 * np.pi, batch=1):
    kw = dict(nx=n, Lx=Lx, dt=dt, stepper=stepper)
    p = gpu.Problem(gpu.GPU(), gpu.OneDAdvectingFlow(u=flow1()), κ=κ, κh=κh, nκh=nκh, T=T, batch=batch, **kw)
    r = oracle.Problem(oracle.OneDAdvectingFlow(u=flow1()), kappa=κ, kappah=κh, nkappah=nκh, **kw)
    return p, r


@pytest.mark.parametrize("n", [16, 32, 64, 128, 256, 512, 1024, 2048, 4096])
@pytest.mark.parametrize("stepper", ["RK4", "ETDRK4"])
def test_1d_fp64(gpu, oracle, n, stepper):
    dt = min(0.002, 0.5 / (0.003 * (n / 2) ** 2))
    p, r = pair1(gpu, oracle, n, stepper=stepper, dt=dt)
    x = gpu.gridpoints(p.grid)
    gpu.set_c(p, ic1(x))
    oracle.set_c(r, ic1(x))
    gpu.stepforward(p, 20)
    oracle.stepforward(r, 20)
    gpu.updatevars(p)
    oracle.updatevars(r)
    assert oracle.rel_l2(p.vars.c, r.vars.c) <= 1e-12
    assert p.clock.step == 20 and abs(p.clock.t - 20 * dt) < 1e-15


@pytest.mark.parametrize("batch", [1, 2, 3])
@pytest.mark.parametrize("T,tol", [(np.float64, 1e-12), (np.float32, 1e-5)])
def test_1d_batch(gpu, oracle, batch, T, tol):
    p, _ = pair1(gpu, oracle, 256, stepper="ETDRK4", T=T, batch=batch, κh=1e-6, nκh=2)
    x = gpu.gridpoints(p.grid)
    cs = np.stack([ic1(x, x0=0.5 * b) for b in range(batch)])
    gpu.set_c(p, cs if batch > 1 else cs[0])
    gpu.stepforward(p, 30)
    gpu.updatevars(p)
    got = p.vars.c.reshape(batch, -1)
    for b in range(batch):
        _, r = pair1(gpu, oracle, 256, stepper="ETDRK4", κh=1e-6, nκh=2)
        oracle.set_c(r, cs[b])
        oracle.stepforward(r, 30)
        oracle.updatevars(r)
        assert oracle.rel_l2(got[b], r.vars.c) <= tol


def test_1d_calcN_and_sol(gpu, oracle):
    p, r = pair1(gpu, oracle, 512)
    x = gpu.gridpoints(p.grid)
    c = ic1(x)
    gpu.set_c(p, c)
    oracle.set_c(r, c)
    sol = p.sol
    assert oracle.rel_l2(sol, r.sol) <= 1e-14
    N = p.calcN(sol)
    Nr = np.zeros_like(r.sol)
    oracle.calcN(Nr, r.sol, 0.0, r.clock, r.params, r.grid)
    assert oracle.rel_l2(N, Nr) <= 1e-13
    # set_sol / get_sol round trip and the state after it
    p.sol = 2 * sol
    assert np.array_equal(p.sol, 2 * sol)
    gpu.updatevars(p)
    assert oracle.rel_l2(p.vars.c, 2 * c) <= 1e-14


def test_1d_fp32_k0_mode(gpu, oracle):
    """FP32 1D with uniform damping (nκh = 0): the mean follows the FP64 oracle.

    The (0,0) state is FP64, but in 1D its right-hand side N(0) = -sum(u c_x)
    is not zero (u varies along x): it is summed in FP64 from FP32 products,
    so its error is that of the FP32 c_x -- about 1e-9 of the mean after 300
    steps here, where an FP32 (0,0) state would drift by ~1e-6."""
    p, r = pair1(gpu, oracle, 256, stepper="RK4", T=np.float32, κh=0.5, nκh=0)
    x = gpu.gridpoints(p.grid)
    c = 1.0 + ic1(x)
    gpu.set_c(p, c)
    oracle.set_c(r, c)
    gpu.stepforward(p, 300)
    oracle.stepforward(r, 300)
    gpu.updatevars(p)
    oracle.updatevars(r)
    r0 = r.sol[0].real
    assert abs(p.sol[0].real - r0) <= 5e-9 * abs(r0)
    assert abs(p.vars.c.sum() - r0) <= 5e-9 * abs(r0)
    assert oracle.rel_l2(p.vars.c, r.vars.c) <= 1e-5


def test_1d_timevarying(gpu, oracle):
    u = lambda x, t: 0.3 + 0.2 * np.sin(x - t)  # noqa: E731
    kw = dict(nx=128, Lx=2 * np.pi, dt=0.005, stepper="RK4")
    p = gpu.Problem(gpu.GPU(), gpu.OneDAdvectingFlow(u=u, steadyflow=False), κ=0.01, **kw)
    r = oracle.Problem(oracle.OneDAdvectingFlow(u=u, steadyflow=False), kappa=0.01, **kw)
    x = gpu.gridpoints(p.grid)
    gpu.set_c(p, ic1(x))
    oracle.set_c(r, ic1(x))
    gpu.stepforward(p, 40)
    oracle.stepforward(r, 40)
    gpu.updatevars(p)
    oracle.updatevars(r)
    assert oracle.rel_l2(p.vars.c, r.vars.c) <= 1e-12


def test_1d_autotune_keeps_state(gpu, oracle):
    p, _ = pair1(gpu, oracle, 1024, batch=4)
    x = gpu.gridpoints(p.grid)
    gpu.set_c(p, np.stack([ic1(x, 0.1 * b) for b in range(4)]))
    gpu.stepforward(p, 2)
    before = p.sol
    t = p.autotune(trial_steps=2, force=True)
    assert t["branches"] == 1 and t["ms_per_step"] > 0
    assert np.array_equal(p.sol, before)


@pytest.mark.parametrize("stepper", ["RK4", "ETDRK4"])
def test_golden_line256_400_steps(gpu, stepper):
    """400 FP64 steps of the 1D golden workload against the committed fixture."""
    from pathlib import Path
    g = np.load(Path(__file__).resolve().parent / "golden" / "line256.npz")
    p = gpu.Problem(gpu.GPU(), gpu.OneDAdvectingFlow(u=lambda x: 0.4 + 0.2 * np.cos(x)), nx=256, κ=1e-3, dt=0.005,
                    stepper=stepper)
    gpu.set_c(p, g["c0"])
    gpu.stepforward(p, 400)
    gpu.updatevars(p)
    c = g[f"c400_{stepper}"]
    assert np.linalg.norm(p.vars.c - c) / np.linalg.norm(c) <= 1e-10
    assert p.clock.step == 400
