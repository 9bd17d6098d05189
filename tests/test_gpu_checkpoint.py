"""Checkpoint / resume of a solve: the state between steps is ``sol`` (with
the FP64 k = 0 mode of FP32 problems) and the clock, which the reference's
JLD2 output records (FourierFlows ``Output``/``saveoutput``; the examples
save ``sol`` and ``clock.t``).  A solve saved after n steps and resumed in a
fresh problem continues bit-identically to the solve that never stopped.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _flow(gpu, dim, steady=True):
    if dim == 1:
        return gpu.OneDAdvectingFlow(u=lambda x: 0.5 + 0.3 * np.sin(x))
    if dim == 3:
        return gpu.ThreeDAdvectingFlow(u=lambda x, y, z: np.sin(z), v=lambda x, y, z: np.cos(z),
                                       w=lambda x, y, z: np.sin(y))
    if steady:
        return gpu.TwoDAdvectingFlow(u=lambda x, y: np.cos(x) * np.sin(y), v=lambda x, y: -np.sin(x) * np.cos(y))
    return gpu.TwoDAdvectingFlow(u=lambda x, y, t: np.cos(x + 0.5 * t) * np.sin(y),
                                 v=lambda x, y, t: -np.sin(x + 0.5 * t) * np.cos(y), steadyflow=False)


def _make(gpu, dim, n, stepper, T, batch=1, steady=True):
    return gpu.Problem(gpu.GPU(), _flow(gpu, dim, steady), nx=n, κ=2e-3, η=1e-3, dt=0.004, stepper=stepper,
                       T=T, batch=batch)


def _ic(gpu, p, batch):
    pts = gpu.gridpoints(p.grid)
    pts = pts if isinstance(pts, tuple) else (pts,)
    c = np.exp(-sum((a - 0.4) ** 2 for a in pts) / 0.3) + 0.2 * np.cos(2 * pts[0])
    return np.stack([c * (1 + 0.1 * j) for j in range(batch)]) if batch > 1 else c


@pytest.mark.parametrize("dim,n,stepper,T,batch,steady", [
    (2, 128, "ETDRK4", np.float64, 1, True),
    (2, 128, "RK4", np.float32, 3, True),
    (2, 64, "ETDRK4", np.float64, 1, False),
    (3, 32, "ETDRK4", np.float32, 1, True),
    (1, 256, "FilteredRK4", np.float64, 2, True),
    (2, 128, "FilteredETDRK4", np.float32, 2, True),  # the compensated pair through the filter
])
def test_resume_is_bit_identical(gpu, tmp_path, dim, n, stepper, T, batch, steady):
    a = _make(gpu, dim, n, stepper, T, batch, steady)
    gpu.set_c(a, _ic(gpu, a, batch))
    gpu.stepforward(a, 7)
    ck = tmp_path / "state.npz"
    t7 = a.clock.t
    a.save_state(ck)
    gpu.stepforward(a, 9)
    gpu.updatevars(a)

    b = _make(gpu, dim, n, stepper, T, batch, steady)
    b.load_state(ck)
    assert b.clock.step == 7 and b.clock.t == t7
    gpu.stepforward(b, 9)
    gpu.updatevars(b)
    assert a.clock.step == b.clock.step == 16 and a.clock.t == b.clock.t
    assert np.array_equal(a.sol, b.sol)
    assert np.array_equal(a.vars.c, b.vars.c)


def test_checkpoint_must_match_problem(gpu, tmp_path):
    a = _make(gpu, 2, 64, "RK4", np.float64)
    ck = tmp_path / "state.npz"
    a.save_state(ck)
    for kw in (dict(n=32, stepper="RK4", T=np.float64), dict(n=64, stepper="ETDRK4", T=np.float64),
               dict(n=64, stepper="RK4", T=np.float32)):
        b = _make(gpu, 2, kw["n"], kw["stepper"], kw["T"])
        with pytest.raises(ValueError):
            b.load_state(ck)


@pytest.mark.parametrize("kw", [dict(κ=5e-3), dict(η=2e-3), dict(Lx=4.0), dict(κh=1e-8, nκh=2)])
def test_checkpoint_of_other_physics_refused(gpu, tmp_path, kw):
    """A checkpoint written for another domain length or diffusivity is
    refused, not continued with physics that do not match."""
    a = _make(gpu, 2, 64, "RK4", np.float64)
    ck = tmp_path / "state.npz"
    a.save_state(ck)
    args = dict(nx=64, κ=2e-3, η=1e-3, dt=0.004, stepper="RK4", T=np.float64)
    args.update(kw)
    b = gpu.Problem(gpu.GPU(), _flow(gpu, 2), **args)
    with pytest.raises(ValueError):
        b.load_state(ck)


def test_output_snapshots_of_a_solve(gpu, oracle, tmp_path):
    """The reference example's output loop (Output with get_concentration,
    saveproblem, saveoutput every 50 steps; examples/onedim_gaussiandiffusion.jl:74-88)
    on a 1D diffusion solve: every stored snapshot equals the oracle's field at
    that step."""
    n, nsteps, every = 128, 200, 50
    p = gpu.Problem(gpu.GPU(), gpu.OneDAdvectingFlow(u=lambda x: 0.0 * x), nx=n, Lx=2 * np.pi, κ=0.01, dt=0.02)
    r = oracle.Problem(oracle.OneDAdvectingFlow(u=lambda x: 0.0 * x), nx=n, Lx=2 * np.pi, kappa=0.01, dt=0.02)
    x = gpu.gridpoints(p.grid)
    c0 = 0.1 * np.exp(-x ** 2 / (2 * 0.1 ** 2))
    gpu.set_c(p, c0)
    oracle.set_c(r, c0)
    out = gpu.Output(p, tmp_path / "advection-diffusion1D.jld2", ("concentration", gpu.get_concentration))
    gpu.saveproblem(out)
    expect = {}
    while p.clock.step <= nsteps:
        if p.clock.step % every == 0:
            gpu.saveoutput(out)
            oracle.updatevars(r)
            expect[p.clock.step] = r.vars.c.copy()
        gpu.stepforward(p)
        oracle.stepforward(r)
    f = gpu.jldopen(out.path)
    steps = sorted(int(k) for k in f["snapshots/t"].keys())
    assert steps == [0, 50, 100, 150, 200]
    for i in steps:
        assert f[f"snapshots/t/{i}"] == pytest.approx(0.02 * i, abs=1e-12)
        assert oracle.rel_l2(f[f"snapshots/concentration/{i}"], expect[i]) <= 1e-12
    assert np.array_equal(f["grid/x"], x)
    f.close()
