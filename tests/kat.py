"""The reference's known-answer tests (test/test_traceradvectiondiffusion.jl)
written once against the API shared by the package and the oracle.

``api`` is either the package (GPU) or the oracle module; both expose
``Problem``, ``TwoDAdvectingFlow``/``ThreeDAdvectingFlow``, ``set_c``,
``stepforward``, ``updatevars``.  Each function returns
``(rel_err, rtol)`` where ``rtol`` is the reference's own tolerance
(``isapprox(cfinal, vs.c, rtol = n*nsteps*1e-12)``).
"""
import numpy as np


def _make(api, dev, flow, **kw):
    if dev is None:  # oracle
        kw = {("kappa" if k == "κ" else k): v for k, v in kw.items()}
        return api.Problem(flow, **kw)
    return api.Problem(dev, flow, **kw)


def _pts(api, prob):
    g = prob.grid
    if hasattr(api, "gridpoints"):
        return api.gridpoints(g)
    return g.gridpoints()


def _rel(a, b):
    a = np.asarray(a).ravel(); b = np.asarray(b).ravel()
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(a), np.linalg.norm(b)))


def _x1(api, prob):
    x = _pts(api, prob)
    return x[0] if isinstance(x, tuple) else x


def constvel1D(api, dev, stepper="RK4", dt=1e-2, nsteps=40):
    """test_constvel1D (:8-33): a Gaussian carried by u = 0.05 on 128 points."""
    uvel, s = 0.05, 0.1
    prob = _make(api, dev, api.OneDAdvectingFlow(u=lambda x: uvel), nx=128, Lx=2 * np.pi, κ=0.0, dt=dt,
                 stepper=stepper)
    x = _x1(api, prob)
    f = lambda x: 0.1 * np.exp(-x ** 2 / (2 * s ** 2))
    api.set_c(prob, f(x)); api.stepforward(prob, nsteps); api.updatevars(prob)
    return _rel(f(x - uvel * nsteps * dt), prob.vars.c), 128 * nsteps * 1e-12


def timedependentvel1D(api, dev, stepper="RK4", dt=0.002, tfinal=0.1, uvel=0.05):
    """test_timedependentvel1D (:42-72): u(t) = uvel t + uvel dt/2, frozen at clock.t per step."""
    nsteps = round(tfinal / dt)
    flow = api.OneDAdvectingFlow(u=lambda x, t: uvel * t + uvel * dt / 2, steadyflow=False)
    prob = _make(api, dev, flow, nx=128, Lx=2 * np.pi, κ=0.0, dt=dt, stepper=stepper)
    x = _x1(api, prob)
    s = 0.2
    f = lambda x: 0.1 * np.exp(-x ** 2 / (2 * s ** 2))
    api.set_c(prob, f(x)); api.stepforward(prob, nsteps); api.updatevars(prob)
    tf = nsteps * dt
    return _rel(f(x - 0.5 * uvel * tf ** 2), prob.vars.c), 128 * nsteps * 1e-12


def diffusion1D(api, dev, stepper="RK4", dt=0.005, tfinal=0.1, steadyflow=True):
    """test_diffusion1D (:232-262): heat kernel with variance 2 kappa t + 0.1 (the
    reference's sigma(t)^2), amplitude 0.1 / sigma(t)."""
    nsteps = round(tfinal / dt)
    κ = 0.01
    prob = _make(api, dev, api.OneDAdvectingFlow(steadyflow=steadyflow), nx=128, Lx=2 * np.pi, κ=κ, dt=dt,
                 stepper=stepper)
    x = _x1(api, prob)
    sig = lambda t: np.sqrt(2 * κ * t + 0.1)
    f = lambda x, t: (0.1 / sig(t)) * np.exp(-x ** 2 / (2 * sig(t) ** 2))
    api.set_c(prob, f(x, 0.0)); api.stepforward(prob, nsteps); api.updatevars(prob)
    return _rel(f(x, nsteps * dt), prob.vars.c), 128 * nsteps * 1e-12


def constvel2D(api, dev, stepper="RK4", dt=1e-2, nsteps=40):
    """test_constvel2D (:79-106)."""
    nx, Lx, uvel, vvel = 128, 2 * np.pi, 0.2, 0.1
    flow = api.TwoDAdvectingFlow(u=lambda x, y: uvel, v=lambda x, y: vvel)
    prob = _make(api, dev, flow, nx=nx, Lx=Lx, κ=0.0, dt=dt, stepper=stepper)
    x, y = _pts(api, prob)
    s = 0.1
    f = lambda x, y: 0.1 * np.exp(-(x ** 2 + y ** 2) / (2 * s ** 2))
    api.set_c(prob, f(x, y)); api.stepforward(prob, nsteps); api.updatevars(prob)
    tf = nsteps * dt
    return _rel(f(x - uvel * tf, y - vvel * tf), prob.vars.c), nx * nx * nsteps * 1e-12


def timedependentvel2D(api, dev, stepper="RK4", dt=0.002, tfinal=0.1, uvel=0.5, av=0.5, **extra):
    """test_timedependentvel2D (:116-145): v(t) = αv t + αv dt/2, frozen at clock.t per step."""
    nsteps = round(tfinal / dt)
    flow = api.TwoDAdvectingFlow(u=lambda x, y, t: uvel, v=lambda x, y, t: av * t + av * dt / 2, steadyflow=False)
    prob = _make(api, dev, flow, nx=128, Lx=2 * np.pi, κ=0.0, dt=dt, stepper=stepper, **extra)
    x, y = _pts(api, prob)
    s = 0.2
    f = lambda x, y: 0.1 * np.exp(-(x ** 2 + y ** 2) / (2 * s ** 2))
    api.set_c(prob, f(x, y)); api.stepforward(prob, nsteps); api.updatevars(prob)
    tf = nsteps * dt
    return _rel(f(x - uvel * tf, y - 0.5 * av * tf ** 2), prob.vars.c), 128 * 128 * nsteps * 1e-12


def diffusion2D(api, dev, stepper="RK4", dt=0.005, tfinal=0.1, steadyflow=True):
    """test_diffusion2D (:272-301)."""
    nsteps = round(tfinal / dt)
    κ = 0.01
    prob = _make(api, dev, api.TwoDAdvectingFlow(steadyflow=steadyflow), nx=128, Lx=2 * np.pi, κ=κ, dt=dt,
                 stepper=stepper)
    x, y = _pts(api, prob)
    s = 0.1
    api.set_c(prob, 0.1 * np.exp(-(x ** 2 + y ** 2) / (2 * s ** 2)))
    api.stepforward(prob, nsteps); api.updatevars(prob)
    tf = nsteps * dt
    st = np.sqrt(2 * κ * tf + s ** 2)
    cf = 0.1 * (s ** 2 / st ** 2) * np.exp(-(x ** 2 + y ** 2) / (2 * st ** 2))
    return _rel(cf, prob.vars.c), 128 * 128 * nsteps * 1e-12


def hyperdiffusion(api, dev, stepper="RK4", dt=0.005, tfinal=0.1):
    """test_hyperdiffusion (:400-439): κ=η=0, κh=0.01, nκh=1."""
    nsteps = round(tfinal / dt)
    κh = 0.01
    kw = dict(nx=128, Lx=2 * np.pi, κ=0.0, η=0.0, dt=dt, stepper=stepper)
    if dev is None:
        kw.update(eta=kw.pop("η"), kappah=κh, nkappah=1)
    else:
        kw.update(κh=κh, nκh=1)
    prob = _make(api, dev, api.TwoDAdvectingFlow(u=lambda x, y: 0.0, v=lambda x, y: 0.0), **kw)
    x, y = _pts(api, prob)
    s = 0.1
    api.set_c(prob, 0.1 * np.exp(-(x ** 2 + y ** 2) / (2 * s ** 2)))
    api.stepforward(prob, nsteps); api.updatevars(prob)
    tf = nsteps * dt
    st = np.sqrt(2 * κh * tf + s ** 2)
    cf = 0.1 * s ** 2 / st ** 2 * np.exp(-(x ** 2 + y ** 2) / (2 * st ** 2))
    return _rel(cf, prob.vars.c), 128 * 128 * nsteps * 1e-12


def diffusion_multilayerqg(api, dev, stepper="RK4", dt=0.005, tfinal=0.1):
    """test_diffusion_multilayerqg (:303-351): a MultiLayerQG problem at rest
    (q = 0, U = 0; 2 layers on 128², stepped to the tracer release time 50 dt),
    each layer's tracer diffusing a Gaussian with κ = η = 0.01; the reference
    checks both layers against the heat kernel at n²·nsteps·1e-12."""
    nsteps = round(tfinal / dt)
    nl, n, L, κ, s = 2, 128, 2 * np.pi, 0.01, 0.1
    if dev is None:
        prob = api.MultiLayerProblem(nx=n, Lx=L, nlayers=nl, dt=dt, kappa=κ, stepper=stepper)
        prob.set_layer_flows(np.zeros((nl, n, n)), np.zeros((nl, n, n)), np.zeros(nl))
        x, y = prob.grid.gridpoints()
    else:
        released = []
        mq = api.MultiLayerQGFlow(nx=n, Lx=L, nlayers=nl, dt=dt, U=np.zeros(nl),
                                  step_until=lambda m, t: released.append(t))  # the QG state stays at rest
        prob = api.Problem(mq, κ=κ, stepper=stepper, tracer_release_time=50 * dt)
        assert released == [50 * dt] and prob.clock.t == 0.0
        x, y = api.gridpoints(prob.grid)
    c0 = 0.1 * np.exp(-(x ** 2 + y ** 2) / (2 * s ** 2))  # one 2D field: set_c! repeats it over the layers
    if dev is None:
        prob.set_c(c0); prob.stepforward(nsteps); prob.updatevars()
        c = prob.c
    else:
        api.set_c(prob, c0); api.stepforward(prob, nsteps); api.updatevars(prob)
        c = prob.vars.c
    tf = nsteps * dt
    st = np.sqrt(2 * κ * tf + s ** 2)
    cf = 0.1 * (s ** 2 / st ** 2) * np.exp(-(x ** 2 + y ** 2) / (2 * st ** 2))
    return max(_rel(cf, c[j]) for j in range(nl)), n * n * nsteps * 1e-12


def constvel3D(api, dev, stepper="RK4", dt=1e-2, nsteps=40, n=128):
    """test_constvel3D (:155-182)."""
    uvel, vvel, wvel = 0.2, 0.1, 0.05
    flow = api.ThreeDAdvectingFlow(u=lambda x, y, z: uvel, v=lambda x, y, z: vvel, w=lambda x, y, z: wvel)
    prob = _make(api, dev, flow, nx=n, Lx=2 * np.pi, κ=0.0, dt=dt, stepper=stepper)
    x, y, z = _pts(api, prob)
    s = 0.1
    f = lambda x, y, z: 0.1 * np.exp(-(x ** 2 + y ** 2 + z ** 2) / (2 * s ** 2))
    api.set_c(prob, f(x, y, z)); api.stepforward(prob, nsteps); api.updatevars(prob)
    tf = nsteps * dt
    return _rel(f(x - uvel * tf, y - vvel * tf, z - wvel * tf), prob.vars.c), n ** 3 * nsteps * 1e-12


def timedependentvel3D(api, dev, stepper="RK4", dt=0.002, tfinal=0.1, uvel=0.5, av=0.5, wvel=0.5, n=128):
    """test_timedependentvel3D (:192-224)."""
    nsteps = round(tfinal / dt)
    flow = api.ThreeDAdvectingFlow(u=lambda x, y, z, t: uvel, v=lambda x, y, z, t: av * t + av * dt / 2,
                                   w=lambda x, y, z, t: wvel, steadyflow=False)
    prob = _make(api, dev, flow, nx=n, Lx=2 * np.pi, κ=0.0, dt=dt, stepper=stepper)
    x, y, z = _pts(api, prob)
    s = 0.2
    f = lambda x, y, z: 0.1 * np.exp(-(x ** 2 + y ** 2 + z ** 2) / (2 * s ** 2))
    api.set_c(prob, f(x, y, z)); api.stepforward(prob, nsteps); api.updatevars(prob)
    tf = nsteps * dt
    return _rel(f(x - uvel * tf, y - 0.5 * av * tf ** 2, z - wvel * tf), prob.vars.c), n ** 3 * nsteps * 1e-12


def diffusion3D(api, dev, stepper="RK4", dt=0.005, tfinal=0.1, steadyflow=True, n=64):
    """test_diffusion3D (:363-392); the reference uses rtol n³·nsteps·1e-10 here."""
    nsteps = round(tfinal / dt)
    κ = 0.01
    prob = _make(api, dev, api.ThreeDAdvectingFlow(steadyflow=steadyflow), nx=n, Lx=2 * np.pi, κ=κ, dt=dt,
                 stepper=stepper)
    x, y, z = _pts(api, prob)
    s = 0.1
    api.set_c(prob, 0.1 * np.exp(-(x ** 2 + y ** 2 + z ** 2) / (2 * s ** 2)))
    api.stepforward(prob, nsteps); api.updatevars(prob)
    tf = nsteps * dt
    st = np.sqrt(2 * κ * tf + s ** 2)
    cf = 0.1 * (s / st) ** 3 * np.exp(-(x ** 2 + y ** 2 + z ** 2) / (2 * st ** 2))
    return _rel(cf, prob.vars.c), n ** 3 * nsteps * 1e-10
