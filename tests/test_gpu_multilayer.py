"""The MultiLayerQG-coupled tracer (src/traceradvectiondiffusion.jl:225-250,
:556-566, :788-804) and the Filtered steppers it defaults to, through the C
ABI against the FP64 oracle.  The QG model itself is outside this package:
layer velocities are synthetic smooth fields, changed between steps as a
stepping MultiLayerQG problem would change them.

Tolerances (relative L2): FP64 1e-12, FP32 1e-5.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def layer_fields(nl, n, L, seed, t=0.0):
    """Divergence-free layer velocities from a few streamfunction modes."""
    rng = np.random.default_rng(seed)
    x = -L / 2 + L / n * np.arange(n)
    Y, X = np.meshgrid(x, x, indexing="ij")
    k = 2 * np.pi / L
    u = np.zeros((nl, n, n))
    v = np.zeros((nl, n, n))
    for j in range(nl):
        for _ in range(3):
            a, b = rng.integers(1, 4, 2)
            ph, amp = rng.uniform(0, 2 * np.pi), rng.uniform(0.3, 1.0)
            arg = k * (a * X + b * Y) + ph + 0.7 * t
            # psi = amp cos(arg): u = -dpsi/dy, v = dpsi/dx
            u[j] += amp * k * b * np.sin(arg)
            v[j] += -amp * k * a * np.sin(arg)
    return u, v


def tracer_ic(nl, n, L):
    x = -L / 2 + L / n * np.arange(n)
    Y, X = np.meshgrid(x, x, indexing="ij")
    return np.stack([np.exp(-((X - 0.4 * j) ** 2 + Y ** 2) / 0.3) for j in range(nl)])


@pytest.mark.parametrize("stepper", ["FilteredRK4", "FilteredETDRK4"])
@pytest.mark.parametrize("T,tol", [(np.float64, 1e-12), (np.float32, 1e-5)])
def test_multilayer_tracer(gpu, oracle, stepper, T, tol):
    nl, n, L, dt = 3, 128, 2 * np.pi, 0.01
    U = np.array([0.3, 0.0, -0.2])
    u0, v0 = layer_fields(nl, n, L, 11)
    mq = gpu.MultiLayerQGFlow(nx=n, Lx=L, nlayers=nl, dt=dt, U=U, u=u0, v=v0)
    p = gpu.Problem(mq, κ=2e-3, η=1e-3, stepper=stepper, T=T)
    assert isinstance(p, gpu.MultiLayerTracerProblem) and p.nlayers == nl
    r = oracle.MultiLayerProblem(nx=n, Lx=L, nlayers=nl, dt=dt, kappa=2e-3, eta=1e-3, stepper=stepper)
    c0 = tracer_ic(nl, n, L)
    gpu.set_c(p, c0)
    r.set_c(c0)
    for k in range(4):  # the QG state moves between tracer steps
        u, v = layer_fields(nl, n, L, 11, t=0.05 * k)
        mq.vars.u, mq.vars.v = u, v
        r.set_layer_flows(u, v, U)
        gpu.stepforward(p, 5)
        r.stepforward(5)
    gpu.updatevars(p)
    r.updatevars()
    assert oracle.rel_l2(p.vars.c, r.c) <= tol
    assert p.clock.step == 20


def test_multilayer_device_velocities(gpu, oracle):
    """Layer velocities as CUDA tensors (the MultiLayerQG state on the device)."""
    torch = pytest.importorskip("torch")
    nl, n, L, dt = 2, 64, 2 * np.pi, 0.01
    u, v = layer_fields(nl, n, L, 3)
    mq = gpu.MultiLayerQGFlow(nx=n, Lx=L, nlayers=nl, dt=dt, U=[0.1, -0.1],
                              u=torch.from_numpy(u).cuda(), v=torch.from_numpy(v).cuda())
    q = gpu.MultiLayerQGFlow(nx=n, Lx=L, nlayers=nl, dt=dt, U=[0.1, -0.1], u=u, v=v)
    p = gpu.Problem(mq, κ=1e-3, stepper="FilteredRK4")
    h = gpu.Problem(q, κ=1e-3, stepper="FilteredRK4")
    c0 = tracer_ic(nl, n, L)
    gpu.set_c(p, c0)
    gpu.set_c(h, c0)
    gpu.stepforward(p, 10)
    gpu.stepforward(h, 10)
    gpu.updatevars(p)
    gpu.updatevars(h)
    assert np.array_equal(p.vars.c, h.vars.c)


def test_multilayer_arguments(gpu):
    mq = gpu.MultiLayerQGFlow(nx=32, nlayers=2, dt=0.01)
    with pytest.raises(ValueError):
        gpu.Problem(mq, tracer_release_time=-1.0)
    with pytest.raises(NotImplementedError):
        gpu.Problem(mq, tracer_release_time=1.0)
    calls = []
    mq2 = gpu.MultiLayerQGFlow(nx=32, nlayers=2, dt=0.01, step_until=lambda m, t: calls.append(t))
    p = gpu.Problem(mq2, tracer_release_time=0.5)
    assert calls == [0.5] and p.tracer_release_time == 0.5


@pytest.mark.parametrize("dim,stepper", [(1, "FilteredRK4"), (2, "FilteredETDRK4"), (3, "FilteredRK4")])
def test_filtered_steppers(gpu, oracle, dim, stepper):
    """FourierFlows' filter applied after every step, in 1D, 2D and 3D."""
    n = {1: 256, 2: 128, 3: 32}[dim]
    kw = dict(nx=n, dt=0.005, stepper=stepper)
    if dim == 1:
        fl = (gpu.OneDAdvectingFlow(u=lambda x: 0.5 + 0.3 * np.sin(x)),
              oracle.OneDAdvectingFlow(u=lambda x: 0.5 + 0.3 * np.sin(x)))
    elif dim == 2:
        fu, fv = (lambda x, y: np.cos(x) * np.sin(y)), (lambda x, y: -np.sin(x) * np.cos(y))
        fl = (gpu.TwoDAdvectingFlow(u=fu, v=fv), oracle.TwoDAdvectingFlow(u=fu, v=fv))
    else:
        fu, fv, fw = (lambda x, y, z: np.sin(z)), (lambda x, y, z: np.cos(z)), (lambda x, y, z: np.sin(y))
        fl = (gpu.ThreeDAdvectingFlow(u=fu, v=fv, w=fw), oracle.ThreeDAdvectingFlow(u=fu, v=fv, w=fw))
    p = gpu.Problem(gpu.GPU(), fl[0], κ=1e-3, **kw)
    r = oracle.Problem(fl[1], kappa=1e-3, **kw)
    pts = gpu.gridpoints(p.grid)
    pts = pts if isinstance(pts, tuple) else (pts,)
    c0 = np.exp(-sum((a - 0.3) ** 2 for a in pts) / 0.2) + 0.1 * np.cos(3 * pts[0])
    gpu.set_c(p, c0)
    oracle.set_c(r, c0)
    gpu.stepforward(p, 12)
    oracle.stepforward(r, 12)
    gpu.updatevars(p)
    oracle.updatevars(r)
    assert oracle.rel_l2(p.vars.c, r.vars.c) <= 1e-12
    # the filter removes the top of the spectrum: the Nyquist column is ~tol
    assert np.abs(p.sol[..., -1]).max() <= 1e-10 * np.abs(p.sol).max()


def test_multilayer_mean_flow_profile(gpu, oracle):
    """A y-dependent imposed zonal flow U_j(y) per layer (GeophysicalFlows
    takes U as a (ny, nlayers) matrix), host and device layer velocities."""
    torch = pytest.importorskip("torch")
    nl, n, L, dt = 2, 64, 2 * np.pi, 0.01
    u, v = layer_fields(nl, n, L, 5)
    y = -L / 2 + L / n * np.arange(n)
    Uy = np.stack([0.4 * np.sin(y), -0.3 * np.cos(y)])
    r = oracle.MultiLayerProblem(nx=n, Lx=L, nlayers=nl, dt=dt, kappa=1e-3, stepper="FilteredRK4")
    r.set_layer_flows(u, v, Uy)
    c0 = tracer_ic(nl, n, L)
    r.set_c(c0)
    r.stepforward(8)
    r.updatevars()
    for dev in (False, True):
        uu, vv = (torch.from_numpy(u).cuda(), torch.from_numpy(v).cuda()) if dev else (u, v)
        mq = gpu.MultiLayerQGFlow(nx=n, Lx=L, nlayers=nl, dt=dt, U=Uy, u=uu, v=vv)
        p = gpu.Problem(mq, κ=1e-3, stepper="FilteredRK4")
        gpu.set_c(p, c0)
        gpu.stepforward(p, 8)
        gpu.updatevars(p)
        assert oracle.rel_l2(p.vars.c, r.c) <= 1e-12
