"""FP64 k = 0 mode of the FP32 form.

With ``k0_fp64`` (the FP32 default) the conserved (0,0[,0]) mode -- its state,
its stage combinations and its coefficients -- is carried in FP64, N(0,0) is a
compensated FP64 sum, and ``vars.c`` reports that mode's mean.  A uniform
damping (``nκh = 0``: L = -κh for every mode, including k = 0) makes the mean
decay, so the FP32 rounding of an FP32 (0,0) state would show; the checks
compare with the FP64 oracle (``oracle/ptf_oracle.py``).

Tolerances: (0,0) mode and mean, relative 1e-9.  The state is FP64; what is
left is N(0,0) summed from FP32 products, whose rounding (about
eps32 * sqrt(points) * rms(N) per evaluation) random-walks to ~1e-10 relative
over these runs.  An FP32 (0,0) state instead rounds by half an ulp of s(0,0)
every step (~1e-6 relative over 300 steps).  The rest of the field keeps the
FP32 bound 1e-5.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

K0_TOL = 1e-9
FP32_TOL = 1e-5


def cellular2(k=1.0):
    return (lambda x, y: k * np.cos(k * x) * np.sin(k * y), lambda x, y: -k * np.sin(k * x) * np.cos(k * y))


def field2(x, y):
    return 1.0 + np.exp(-((x - 1.0) ** 2 + (y - 2.0) ** 2) / 0.18) + 0.3 * np.cos(2 * x + y)


def run2(gpu, oracle, stepper, k0, n=128, nsteps=300, dt=0.002):
    u, v = cellular2()
    kw = dict(nx=n, dt=dt, stepper=stepper)
    p = gpu.Problem(gpu.GPU(), gpu.TwoDAdvectingFlow(u=u, v=v), κ=1e-3, κh=0.5, nκh=0, T=np.float32,
                    k0_fp64=k0, **kw)
    r = oracle.Problem(oracle.TwoDAdvectingFlow(u=u, v=v), kappa=1e-3, kappah=0.5, nkappah=0, **kw)
    x, y = gpu.gridpoints(p.grid)
    c0 = field2(x, y)
    gpu.set_c(p, c0)
    oracle.set_c(r, c0)
    gpu.stepforward(p, nsteps)
    oracle.stepforward(r, nsteps)
    gpu.updatevars(p)
    oracle.updatevars(r)
    return p, r


@pytest.mark.parametrize("stepper", ["RK4", "ETDRK4"])
def test_k0_mode_2d_decay(gpu, oracle, stepper):
    p, r = run2(gpu, oracle, stepper, True)
    s00, r00 = p.sol[0, 0], r.sol[0, 0]
    assert abs(s00.imag) == 0.0
    assert abs(s00.real - r00.real) <= K0_TOL * abs(r00.real)
    # vars.c carries the FP64 mean
    assert abs(p.vars.c.sum() - r00.real) <= K0_TOL * abs(r00.real)
    assert abs(p.vars.c.mean() - r.vars.c.mean()) <= K0_TOL * abs(r.vars.c.mean())
    assert oracle.rel_l2(p.vars.c, r.vars.c) <= FP32_TOL
    # the rest of the spectrum keeps FP32 accuracy
    assert oracle.rel_l2(p.sol, r.sol) <= FP32_TOL


def test_k0_mode_off_is_plain_fp32(gpu, oracle):
    """k0_fp64=False: all-FP32 state; its (0,0) error is FP32-sized, well above the FP64 mode's."""
    p, r = run2(gpu, oracle, "RK4", False)
    q, _ = run2(gpu, oracle, "RK4", True)
    assert oracle.rel_l2(p.vars.c, r.vars.c) <= FP32_TOL
    r00 = r.sol[0, 0].real
    err_off = abs(p.sol[0, 0].real - r00)
    err_on = abs(q.sol[0, 0].real - r00)
    assert err_off <= 1e-5 * abs(r00)
    assert err_on * 10 < err_off


def test_k0_mode_set_sol_round_trip(gpu, oracle):
    """set_sol/get_sol: (0,0) comes back bit-exact in FP64; the rest is held
    as the compensated FP32 pair s + s_lo (s the FP32 rounding, s_lo that of
    the remainder), which returns every value to within 2^-47 of itself."""
    u, v = cellular2()
    p = gpu.Problem(gpu.GPU(), gpu.TwoDAdvectingFlow(u=u, v=v), nx=64, T=np.float32)
    rng = np.random.default_rng(7)
    sol = rng.standard_normal(p.grid.spec_shape) + 1j * rng.standard_normal(p.grid.spec_shape)
    sol[0, 0] = np.pi * 1e4 + 0.0j
    p.sol = sol
    back = p.sol
    assert back[0, 0] == sol[0, 0]
    rest = back.copy()
    rest[0, 0] = 0
    ref = sol.copy()
    ref[0, 0] = 0
    nz = ref != 0
    assert np.max(np.abs(rest[nz] - ref[nz]) / np.abs(ref[nz])) <= 2.0 ** -47
    # and a second round trip is exact: the pair is canonical
    p.sol = back
    assert np.array_equal(p.sol, back)
    # vars.c: sum of the field equals the FP64 (0,0) mode
    gpu.updatevars(p)
    assert abs(p.vars.c.sum() - sol[0, 0].real) <= 1e-12 * abs(sol[0, 0].real)


def test_k0_mode_batch_and_schedule(gpu, oracle):
    """Per-solve FP64 k = 0 state under batching, groups and stream branches."""
    u, v = cellular2()
    kw = dict(nx=64, dt=0.002, stepper="ETDRK4")
    p = gpu.Problem(gpu.GPU(), gpu.TwoDAdvectingFlow(u=u, v=v), κ=1e-3, κh=0.5, nκh=0, T=np.float32, batch=4, **kw)
    p.set_schedule(solves_per_group=1, branches=2, use_graph=True)
    x, y = gpu.gridpoints(p.grid)
    cs = np.stack([field2(x, y) * (b + 1) for b in range(4)])
    gpu.set_c(p, cs)
    gpu.stepforward(p, 40)
    gpu.updatevars(p)
    sols = p.sol
    for b in range(4):
        r = oracle.Problem(oracle.TwoDAdvectingFlow(u=u, v=v), kappa=1e-3, kappah=0.5, nkappah=0, **kw)
        oracle.set_c(r, cs[b])
        oracle.stepforward(r, 40)
        r00 = r.sol[0, 0].real
        assert abs(sols[b, 0, 0].real - r00) <= K0_TOL * abs(r00)
        assert abs(p.vars.c[b].sum() - r00) <= K0_TOL * abs(r00)


@pytest.mark.parametrize("stepper", ["RK4", "ETDRK4"])
def test_k0_mode_3d_decay(gpu, oracle, stepper):
    A, B, C = 1.0, np.sqrt(2 / 3), np.sqrt(1 / 3)
    u = lambda x, y, z: A * np.sin(z) + C * np.cos(y)  # noqa: E731
    v = lambda x, y, z: B * np.sin(x) + A * np.cos(z)  # noqa: E731
    w = lambda x, y, z: C * np.sin(y) + B * np.cos(x)  # noqa: E731
    kw = dict(nx=32, dt=0.004, stepper=stepper)
    p = gpu.Problem(gpu.GPU(), gpu.ThreeDAdvectingFlow(u=u, v=v, w=w), κ=1e-3, κh=0.5, nκh=0, T=np.float32, **kw)
    r = oracle.Problem(oracle.ThreeDAdvectingFlow(u=u, v=v, w=w), kappa=1e-3, kappah=0.5, nkappah=0, **kw)
    x, y, z = gpu.gridpoints(p.grid)
    c0 = 2.0 + np.cos(x) * np.sin(2 * y) + 0.5 * np.exp(-((z - 3.0) ** 2))
    gpu.set_c(p, c0)
    oracle.set_c(r, c0)
    gpu.stepforward(p, 60)
    oracle.stepforward(r, 60)
    gpu.updatevars(p)
    oracle.updatevars(r)
    r00 = r.sol[0, 0, 0].real
    assert abs(p.sol[0, 0, 0].real - r00) <= K0_TOL * abs(r00)
    assert abs(p.vars.c.sum() - r00) <= K0_TOL * abs(r00)
    assert oracle.rel_l2(p.vars.c, r.vars.c) <= FP32_TOL
