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
