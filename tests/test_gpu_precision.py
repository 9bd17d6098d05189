"""FP32 accuracy over long runs: the compensated state and the exact
twiddles against the FP64 oracle.

An FP32 handle holds its stepper state as a pair of FP32 values and adds each
step's increment to the pair with a two-sum, so rounding the state costs
nothing per step; its transforms use only correctly rounded twiddles.  These
tests pin what that buys:

* pure diffusion (no flow) for 3000 ETDRK4 steps: every mode is s0 E^n, so
  an FP32 state that rounds every step random-walks to a few 1e-6; the
  compensated state follows the oracle to the FP32 tables' rounding;
* the 1024^2 cellular-flow workload of the benchmark (ETDRK4, kappa = eta =
  1e-4, kappah = 1e-12, nkappah = 2) over its configured 1000 steps: within
  the 1e-5 relative L2 that FP32 results are held to (an FP32 state with
  twiddles built as products of rounded powers reached 1.5e-5).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _gauss(x, y, x0=np.pi / 2, y0=np.pi / 2, s=0.2):
    return np.exp(-((x - x0) ** 2 + (y - y0) ** 2) / (2 * s ** 2))


def test_fp32_pure_diffusion_3000_steps(gpu, oracle):
    n, steps, dt = 128, 3000, 0.01
    zero = lambda x, y: 0.0 * x  # noqa: E731
    kw = dict(nx=n, Lx=2 * np.pi, dt=dt, stepper="ETDRK4")
    p = gpu.Problem(gpu.GPU(), gpu.TwoDAdvectingFlow(u=zero, v=zero), κ=2e-4, η=1e-4, T=np.float32, **kw)
    r = oracle.Problem(oracle.TwoDAdvectingFlow(u=zero, v=zero), kappa=2e-4, eta=1e-4, **kw)
    x, y = gpu.gridpoints(p.grid)
    c0 = _gauss(x, y, s=0.3) + 0.1 * np.cos(3 * x + 2 * y)
    gpu.set_c(p, c0)
    oracle.set_c(r, c0)
    gpu.stepforward(p, steps)
    oracle.stepforward(r, steps)
    gpu.updatevars(p)
    oracle.updatevars(r)
    err = oracle.rel_l2(p.vars.c, r.vars.c)
    assert err <= 5e-7, err
    # the state itself (sol), not only the field read back in FP32
    assert oracle.rel_l2(p.sol, r.sol) <= 5e-7


def test_fp32_benchmark_workload_1000_steps(gpu, oracle):
    n, steps, dt = 1024, 1000, 5e-4
    u = lambda x, y: 4.0 * np.cos(4 * x) * np.sin(4 * y)  # noqa: E731
    v = lambda x, y: -4.0 * np.sin(4 * x) * np.cos(4 * y)  # noqa: E731
    kw = dict(nx=n, Lx=2 * np.pi, dt=dt, stepper="ETDRK4")
    p = gpu.Problem(gpu.GPU(), gpu.TwoDAdvectingFlow(u=u, v=v), κ=1e-4, η=1e-4, κh=1e-12, nκh=2, T=np.float32,
                    **kw)
    r = oracle.Problem(oracle.TwoDAdvectingFlow(u=u, v=v), kappa=1e-4, eta=1e-4, kappah=1e-12, nkappah=2, **kw)
    x, y = gpu.gridpoints(p.grid)
    c0 = _gauss(x, y)
    m0 = float(c0.sum())
    gpu.set_c(p, c0)
    oracle.set_c(r, c0)
    gpu.stepforward(p, steps)
    oracle.stepforward(r, steps)
    gpu.updatevars(p)
    oracle.updatevars(r)
    assert oracle.rel_l2(p.vars.c, r.vars.c) <= 1e-5
    assert abs(p.vars.c.sum() / m0 - r.vars.c.sum() / m0) <= 1e-8
