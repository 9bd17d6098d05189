"""Batched form (ptf_batch_*): many independent 2D solves stepped together
(per stage a row launch and a column launch over all solves' work items, or
one persistent kernel), against single-solve handles and the oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def gauss(n, x0, y0, s, L=2 * np.pi):
    x = -L / 2 + L / n * np.arange(n)
    Y, X = np.meshgrid(x, x, indexing="ij")
    dx = (X - x0 + L / 2) % L - L / 2
    dy = (Y - y0 + L / 2) % L - L / 2
    return np.exp(-(dx ** 2 + dy ** 2) / (2 * s ** 2))


def cellular_arrays(n, k=1, U=1.0, L=2 * np.pi):
    x = -L / 2 + L / n * np.arange(n)
    Y, X = np.meshgrid(x, x, indexing="ij")
    return U * k * np.cos(k * X) * np.sin(k * Y), -U * k * np.sin(k * X) * np.cos(k * Y)


def single(gpu, n, κ, dt, nsteps, c0, u, v, T):
    p = gpu.Problem(gpu.GPU(), gpu.TwoDAdvectingFlow(), nx=n, κ=κ, η=κ, dt=dt, T=T)
    p.set_flow_arrays(u, v)
    gpu.set_c(p, c0)
    gpu.stepforward(p, nsteps)
    gpu.updatevars(p)
    return p.vars.c.copy()


@pytest.mark.parametrize("T,tol", [(np.float64, 1e-12), (np.float32, 1e-5)])
@pytest.mark.parametrize("use_graph", [True, False])
def test_batch_matches_single_handles(gpu, oracle, T, tol, use_graph):
    """Mixed sizes, diffusivities and step counts; each solve equals its own
    single-handle run (FP64 to round-off; FP32 within the FP32 tolerance of
    the FP64 oracle) and stops at its own step count."""
    rng = np.random.default_rng(7)
    b = gpu.BatchedProblem(T=T, use_graph=use_graph, slots_per_bucket=4)
    cases = []
    for i, n in enumerate([64, 128, 64, 256, 128, 64]):
        κ = float(10 ** rng.uniform(-4, -2))
        dt = 0.004
        nsteps = [5, 8, 3, 6, 8, 7][i]
        c0 = gauss(n, *rng.uniform(-3, 3, 2), rng.uniform(0.3, 0.6))
        u, v = cellular_arrays(n, k=1 + i % 2)
        sid = b.add(gpu.SolveSpec(n=n, nsteps=nsteps, dt=dt, kappa=κ), c0, u, v)
        cases.append((sid, n, κ, dt, nsteps, c0, u, v))
    b.step(10)  # every solve stops at its own nsteps
    for sid, n, κ, dt, nsteps, c0, u, v in cases:
        step, t, active = b.status(sid)
        assert step == nsteps and not active and abs(t - nsteps * dt) < 1e-14
        ref = single(gpu, n, κ, dt, nsteps, c0, u, v, np.float64)
        assert oracle.rel_l2(b.get_c(sid), ref) <= tol


@pytest.mark.parametrize("time_mode", ["clock", "stage"])
@pytest.mark.parametrize("T,tol", [(np.float64, 1e-12), (np.float32, 1e-5)])
def test_batch_cellular_time_varying_vs_oracle(gpu, oracle, time_mode, T, tol):
    """ψ = cos(x + 0.3 sin t) cos y evaluated on the device at clock.t (the
    reference's rule) or at every RK4 stage time (the batched ensemble's
    configuration), against the oracle with the same rule."""
    eps, om = 0.3, 1.0
    u = lambda x, y, t: np.cos(x + eps * np.sin(om * t)) * np.sin(y)
    v = lambda x, y, t: -np.sin(x + eps * np.sin(om * t)) * np.cos(y)
    b = gpu.BatchedProblem(T=T)
    ids = []
    for n, κ in ((64, 1e-3), (128, 3e-3)):
        c0 = gauss(n, 0.5, -0.7, 0.4)
        spec = gpu.SolveSpec(n=n, nsteps=12, dt=0.005, kappa=κ, flow="cellular", time_mode=time_mode,
                             U=1.0, eps=eps, omega=om, Kx=1, Ky=1)
        ids.append((b.add(spec, c0), n, κ, c0))
    b.step(12)
    for sid, n, κ, c0 in ids:
        r = oracle.Problem(oracle.TwoDAdvectingFlow(u=u, v=v, steadyflow=False), nx=n, kappa=κ, dt=0.005,
                           stage_time=(time_mode == "stage"))
        oracle.set_c(r, c0)
        oracle.stepforward(r, 12)
        oracle.updatevars(r)
        assert oracle.rel_l2(b.get_c(sid), r.vars.c) <= tol


def test_batch_admission_between_steps_and_reuse(gpu):
    """A solve added after others have stepped, and one placed in a freed
    slot, give the same result as a solve run alone."""
    n, dt = 64, 0.004
    u, v = cellular_arrays(n)
    c0 = gauss(n, 1.0, 0.2, 0.5)
    spec = gpu.SolveSpec(n=n, nsteps=6, dt=dt, kappa=1e-3)
    alone = gpu.BatchedProblem(T=np.float64)
    a = alone.add(spec, c0, u, v)
    alone.step(6)
    ref = alone.get_c(a)
    b = gpu.BatchedProblem(T=np.float64, slots_per_bucket=2)
    first = b.add(gpu.SolveSpec(n=n, nsteps=20, dt=dt, kappa=5e-3), gauss(n, -1, 0, 0.3), u, v)
    b.step(3)
    late = b.add(spec, c0, u, v)  # admitted mid-flight
    b.step(6)
    assert np.array_equal(b.get_c(late), ref)
    b.remove(late)
    again = b.add(spec, c0, u, v)  # reuses the freed slot
    b.step(6)
    assert np.array_equal(b.get_c(again), ref)
    assert b.status(first)[0] == 15


def test_batch_rejects_bad_descriptions(gpu):
    from ptf_gb300._lib import PtfArgumentError
    b = gpu.BatchedProblem()
    with pytest.raises(PtfArgumentError):
        b.add(gpu.SolveSpec(n=100, nsteps=1, dt=0.01), np.zeros((100, 100)), np.zeros((100, 100)), np.zeros((100, 100)))
    with pytest.raises(PtfArgumentError):
        b.add(gpu.SolveSpec(n=64, nsteps=1, dt=0.01), np.zeros((64, 64)))  # array flow without arrays


def test_batch_memory_budget(gpu):
    from ptf_gb300._lib import PtfError
    b = gpu.BatchedProblem(T=np.float32, memory_budget=64 << 20, slots_per_bucket=64)
    n = 256
    u, v = cellular_arrays(n)
    added = 0
    with pytest.raises(MemoryError):
        for i in range(1000):
            b.add(gpu.SolveSpec(n=n, nsteps=1, dt=0.001, kappa=1e-3), gauss(n, 0, 0, 0.4), u, v)
            added += 1
    assert 0 < added < 1000
    assert b.info()["device_bytes"] <= 64 << 20


@pytest.mark.parametrize("T,tol", [(np.float64, 1e-13), (np.float32, 1e-6)])
def test_persistent_and_item_launches_agree(gpu, oracle, T, tol):
    """The persistent kernel and the two launches per stage run the same item
    bodies: same results for a mixed-size batch with its own step counts."""
    rng = np.random.default_rng(11)
    cases = [(n, steps, gauss(n, *rng.uniform(-2, 2, 2), 0.3)) for n, steps in ((64, 7), (128, 12), (64, 12), (256, 5))]
    out = []
    for persistent in (False, True):
        b = gpu.BatchedProblem(T=T, slots_per_bucket=3, persistent=persistent)
        ids = []
        for n, steps, c0 in cases:
            u, v = cellular_arrays(n, k=2)
            ids.append(b.add(gpu.SolveSpec(n=n, nsteps=steps, dt=0.004, kappa=2e-3, flow="arrays"), c0, u, v))
        b.step(12)
        out.append([b.get_c(i) for i in ids])
        b.close()
    for a, c in zip(*out):
        assert oracle.rel_l2(a, c) <= tol


def _uniform_damping_case(gpu, oracle, n=128, nsteps=300, dt=0.002):
    """Uniform damping (nκh = 0: L = -κh for every mode, k = 0 included) makes
    the mean decay, so an FP32 (0,0) state's rounding would show."""
    u, v = cellular_arrays(n)
    x = -np.pi + 2 * np.pi / n * np.arange(n)
    Y, X = np.meshgrid(x, x, indexing="ij")
    c0 = 1.0 + np.exp(-((X - 1.0) ** 2 + (Y - 2.0) ** 2) / 0.18) + 0.3 * np.cos(2 * X + Y)
    spec = gpu.SolveSpec(n=n, nsteps=nsteps, dt=dt, kappa=1e-3, kappah=0.5, nkappah=0)
    r = oracle.Problem(oracle.TwoDAdvectingFlow(u=lambda *a: u, v=lambda *a: v), nx=n, kappa=1e-3, kappah=0.5,
                       nkappah=0, dt=dt)
    oracle.set_c(r, c0)
    oracle.stepforward(r, nsteps)
    oracle.updatevars(r)
    return spec, c0, u, v, r


def test_batch_k0_mode_mean_vs_oracle(gpu, oracle):
    """FP32 batched solves carry the conserved (0,0) mode in FP64 (k0_mode, the
    default): the mean of the result matches the FP64 oracle to 1e-9 relative
    (the FP64 state leaves only the rounding of N(0,0) summed from FP32
    products), the field keeps the FP32 bound 1e-5; with the mode off the mean
    is FP32-rounded, at least ten times further off."""
    spec, c0, u, v, r = _uniform_damping_case(gpu, oracle)
    errs = {}
    for k0 in (True, False):
        b = gpu.BatchedProblem(T=np.float32, slots_per_bucket=2, k0_mode=k0)
        ids = [b.add(spec, c0, u, v), b.add(spec, c0, u, v)]  # two slots: column 0 of each in its own lines
        b.step(spec.nsteps)
        cs = [b.get_c(i) for i in ids]
        b.close()
        for c in cs:
            assert oracle.rel_l2(c, r.vars.c) <= 1e-5
        errs[k0] = max(abs(c.sum() - r.vars.c.sum()) / abs(r.vars.c.sum()) for c in cs)
    assert errs[True] <= 1e-9
    assert errs[True] * 10 < errs[False]


@pytest.mark.parametrize("n", [64, 256])
def test_batch_k0_mode_sizes_and_persistent(gpu, oracle, n):
    """Every bucket size's column layout (64: a block's lines span two slots)
    and the persistent kernel keep the FP64 mean."""
    spec, c0, u, v, r = _uniform_damping_case(gpu, oracle, n=n, nsteps=120)
    for persistent in (False, True):
        b = gpu.BatchedProblem(T=np.float32, slots_per_bucket=3, persistent=persistent)
        ids = [b.add(spec, c0, u, v) for _ in range(3)]
        b.step(spec.nsteps)
        for i in ids:
            c = b.get_c(i)
            assert abs(c.sum() - r.vars.c.sum()) <= 1e-9 * abs(r.vars.c.sum())
            assert oracle.rel_l2(c, r.vars.c) <= 1e-5
        b.close()
