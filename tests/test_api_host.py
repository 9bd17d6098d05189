"""Host-side behaviour of the Python mirror of the reference API (no GPU)."""
import numpy as np
import pytest


def test_cpu_device_is_refused(pkg):
    with pytest.raises(NotImplementedError):
        pkg.Problem(pkg.CPU(), pkg.TwoDAdvectingFlow())


def test_bad_stepper(pkg):
    with pytest.raises(ValueError):
        pkg.Problem(pkg.GPU(), pkg.TwoDAdvectingFlow(), stepper="Euler")


def test_bad_dtype(pkg):
    with pytest.raises(ValueError):
        pkg.Problem(pkg.GPU(), pkg.TwoDAdvectingFlow(), T=np.int32)


def test_unknown_keyword(pkg):
    with pytest.raises(TypeError):
        pkg.Problem(pkg.GPU(), pkg.TwoDAdvectingFlow(), nsteps=3)


def test_bad_grid_raises_argument_error(pkg):
    from ptf_gb300._lib import PtfArgumentError
    with pytest.raises(PtfArgumentError):
        pkg.Problem(pkg.GPU(), pkg.TwoDAdvectingFlow(), nx=100)


def test_flow_containers_match_reference(pkg):
    f = pkg.TwoDAdvectingFlow()
    u, v, steady = f
    assert u(1.0, 2.0) == 0.0 and v(0.0, 0.0) == 0.0 and steady is True
    f3 = pkg.ThreeDAdvectingFlow(steadyflow=False)
    assert len(list(f3)) == 4 and f3.steadyflow is False
    assert pkg.noflow(np.pi) == 0


def test_grid_matches_oracle(pkg, oracle):
    g = pkg.TwoDGrid(nx=64, Lx=2 * np.pi, ny=32, Ly=3.0)
    o = oracle.Grid(2, 64, 2 * np.pi, 32, 3.0)
    assert np.array_equal(g.x, o.x) and np.array_equal(g.y, o.y)
    assert np.array_equal(g.kr, o.kr.ravel()) and np.array_equal(g.l, o.l.ravel())
    X, Y = pkg.gridpoints(g)
    Xo, Yo = o.gridpoints()
    assert np.array_equal(X, Xo) and np.array_equal(Y, Yo)


def test_one_d_grid_and_gridpoints(pkg, oracle):
    g = pkg.OneDGrid(nx=64, Lx=3.0)
    x = pkg.gridpoints(g)
    assert x.shape == (64,) and g.spec_shape == (33,)
    r = oracle.Grid(1, 64, 3.0)
    assert np.array_equal(x, r.gridpoints()[0])
    assert np.allclose(g.Krsq, r.Krsq)


def test_filtered_steppers_are_accepted_names(pkg):
    """FilteredRK4 / FilteredETDRK4 pass the host checks (the handle itself
    needs a GPU: without one the call gets as far as the device)."""
    from ptf_gb300._lib import PtfArgumentError
    for st in ("FilteredRK4", "FilteredETDRK4"):
        with pytest.raises(Exception) as e:
            pkg.Problem(pkg.GPU(), pkg.TwoDAdvectingFlow(), nx=32, stepper=st)
        assert not isinstance(e.value, (ValueError, PtfArgumentError))


def test_multilayer_dispatch_and_arguments(pkg):
    """Problem(MQGprob; ...) dispatches on a MultiLayerQG-like first argument
    (:225-250) and checks tracer_release_time before touching the device."""
    mq = pkg.MultiLayerQGFlow(nx=32, nlayers=3, dt=0.01, U=[0.1, 0.0, -0.1])
    assert mq.params.nlayers == 3 and mq.vars.u.shape == (3, 32, 32) and mq.clock.dt == 0.01
    assert np.allclose(mq.params.U, [0.1, 0.0, -0.1])
    with pytest.raises(ValueError):
        pkg.Problem(mq, tracer_release_time=-1.0)
    with pytest.raises(NotImplementedError):
        pkg.Problem(mq, tracer_release_time=0.5)  # the stand-in cannot advance itself
    with pytest.raises(TypeError):
        pkg.Problem(mq, nsteps=3)
    seen = []
    mq2 = pkg.MultiLayerQGFlow(nx=32, nlayers=2, dt=0.01, step_until=lambda m, t: seen.append(t))
    with pytest.raises(Exception):  # no GPU here: fails at the device, after stepping the flow
        pkg.Problem(mq2, tracer_release_time=0.25)
    assert seen == [0.25]


def test_tracer_release_is_logged(pkg, caplog):
    """@info "Stepping the flow forward until t = tracer_release_time = ..." (:237)."""
    import logging
    mq = pkg.MultiLayerQGFlow(nx=32, nlayers=2, dt=0.01, step_until=lambda m, t: None)
    with caplog.at_level(logging.INFO, logger="ptf_gb300"):
        with pytest.raises(Exception):  # no GPU here
            pkg.Problem(mq, tracer_release_time=0.25)
    assert "tracer_release_time = 0.25" in caplog.text


def test_device_arrays_are_checked_before_the_library_reads_them(pkg):
    """The library reads exactly the problem's number of float64 values from
    a device pointer: wrong dtype, layout or size is refused on the host
    (checked here on CPU tensors, which take the same checks)."""
    torch = pytest.importorskip("torch")
    from ptf_gb300 import traceradvectiondiffusion as tad
    ok = torch.zeros(3, 8, dtype=torch.float64)
    assert tad._device_array(ok, 24, "u") is ok
    with pytest.raises(ValueError, match="float64"):
        tad._device_array(torch.zeros(24, dtype=torch.float32), 24, "u")
    with pytest.raises(ValueError, match="contiguous"):
        tad._device_array(ok.t(), 24, "u")
    with pytest.raises(ValueError, match="23 values"):
        tad._device_array(torch.zeros(23, dtype=torch.float64), 24, "u")


def test_host_and_device_arrays_are_not_mixed(pkg):
    from ptf_gb300 import traceradvectiondiffusion as tad

    class OnDevice:
        is_cuda = True

    assert tad._all_host_or_device((np.zeros(2), np.zeros(2)), "u, v") is False
    assert tad._all_host_or_device((OnDevice(), OnDevice()), "u, v") is True
    with pytest.raises(ValueError, match="mix"):
        tad._all_host_or_device((np.zeros(2), OnDevice()), "u, v")


def test_multilayer_oracle_repeats_one_field_over_layers(oracle):
    """set_c! of a MultiLayerQG-coupled problem (:861-870) repeats a 2D field."""
    p = oracle.MultiLayerProblem(nx=16, nlayers=3, dt=0.01, kappa=0.01)
    c = np.random.default_rng(0).standard_normal((16, 16))
    p.set_c(c)
    assert all(np.allclose(p.c[j], c, atol=1e-14) for j in range(3))


def test_flow_display(pkg):
    """Base.show of the flow containers (src/traceradvectiondiffusion.jl:110-125)."""
    def cellu(x, y):
        return 0.0
    s = str(pkg.TwoDAdvectingFlow(u=cellu, steadyflow=False)).splitlines()
    assert s[0] == "TwoDAdvectingFlow"
    assert s[1] == "  ├────────── u: cellu" and s[2] == "  ├────────── v: noflow"
    assert s[3] == "  └─ steadyflow: false"
    assert len(str(pkg.ThreeDAdvectingFlow()).splitlines()) == 5
    assert len(str(pkg.OneDAdvectingFlow()).splitlines()) == 3


def test_layer_mean_flow_forms(pkg):
    """MQGprob.params.U: a scalar, one value per layer, or a (nlayers, ny)
    profile U_j(y) (GeophysicalFlows' (ny, nlayers) matrix) added along x."""
    from ptf_gb300 import traceradvectiondiffusion as tad
    per, prof = tad._layer_mean_flow([0.1, -0.2], 2, 8)
    assert np.allclose(per, [0.1, -0.2]) and prof is None
    per, prof = tad._layer_mean_flow(0.3, 2, 8)
    assert np.allclose(per, [0.3, 0.3]) and prof is None
    Uy = np.arange(16.0).reshape(2, 8)
    per, prof = tad._layer_mean_flow(Uy, 2, 8)
    assert per is None and prof.shape == (2, 8, 1) and prof[1, 3, 0] == Uy[1, 3]
    u = np.zeros((2, 8, 4)) + prof  # broadcasts along x
    assert np.all(u[1, 3] == Uy[1, 3])
    with pytest.raises(ValueError):
        tad._layer_mean_flow(np.zeros(5), 2, 8)


def test_oracle_layer_profile_is_u_plus_U_of_y(oracle):
    """The oracle adds a (nlayers, ny) mean-flow profile to u along x (:794)."""
    n, nl = 32, 2
    rng = np.random.default_rng(1)
    u, v = rng.standard_normal((nl, n, n)) * 0.1, rng.standard_normal((nl, n, n)) * 0.1
    y = -np.pi + 2 * np.pi / n * np.arange(n)
    Uy = np.stack([0.5 * np.sin(y), 0.2 * np.cos(2 * y)])
    a = oracle.MultiLayerProblem(nx=n, nlayers=nl, dt=0.01, kappa=1e-3, stepper="RK4")
    b = oracle.MultiLayerProblem(nx=n, nlayers=nl, dt=0.01, kappa=1e-3, stepper="RK4")
    a.set_layer_flows(u, v, Uy)
    b.set_layer_flows(u + Uy[:, :, None], v, None)
    x = -np.pi + 2 * np.pi / n * np.arange(n)
    Y, X = np.meshgrid(y, x, indexing="ij")
    c0 = np.exp(-(X ** 2 + Y ** 2) / 0.5)
    for p in (a, b):
        p.set_c(c0)
        p.stepforward(5)
        p.updatevars()
    assert np.array_equal(a.c, b.c)


def test_solve_spec_maps_to_the_c_descriptor(pkg):
    """SolveSpec -> ptf_solve_desc (no device needed): η defaults to κ, the
    flow and time-mode names map to the ABI's enums."""
    from ptf_gb300 import _lib as L
    d = pkg.SolveSpec(n=256, nsteps=40, dt=0.003, kappa=2e-3, flow="cellular", time_mode="stage", U=0.5, eps=0.3,
                      omega=2.0, Kx=2, Ky=3).desc()
    assert (d.dim, d.n, d.nsteps) == (2, 256, 40) and d.dt == 0.003
    assert d.kappa == 2e-3 and d.eta == 2e-3
    assert d.flow_kind == L.PTF_FLOW_CELLULAR and d.time_mode == L.PTF_STAGE_T
    assert (d.U, d.eps, d.omega, d.Kx, d.Ky) == (0.5, 0.3, 2.0, 2, 3)
    assert abs(d.L - 2 * np.pi) < 1e-15
    d = pkg.SolveSpec(n=64, nsteps=1, dt=0.01, kappa=1e-3, eta=5e-4).desc()
    assert d.eta == 5e-4 and d.flow_kind == L.PTF_FLOW_ARRAYS and d.time_mode == L.PTF_CLOCK_T
    assert pkg.SolveSpec(n=32, nsteps=1, dt=0.1, dim=3).points == 32 ** 3
    with pytest.raises(KeyError):
        pkg.SolveSpec(n=64, nsteps=1, dt=0.01, flow="turbulent").desc()
