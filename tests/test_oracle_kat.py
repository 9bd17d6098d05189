"""Pin the CPU oracle to the reference's own known-answer tests.

Each reference test (test/test_traceradvectiondiffusion.jl, driven by
test/runtests.jl:26-54 with stepper "RK4") is run against the oracle at the
reference's tolerance, and at a much tighter bound that documents how close
the restatement actually lands.
"""
import numpy as np
import pytest

import kat


@pytest.mark.parametrize("name,tight", [
    ("constvel2D", 2e-8), ("timedependentvel2D", 1e-10), ("diffusion2D", 1e-9), ("hyperdiffusion", 1e-9),
])
def test_reference_kat_2d(oracle, name, tight):
    err, rtol = getattr(kat, name)(oracle, None)
    assert err <= rtol, f"{name}: {err:.3e} > reference rtol {rtol:.3e}"
    assert err <= tight


@pytest.mark.parametrize("name,tight", [("constvel1D", 1e-9), ("timedependentvel1D", 1e-9), ("diffusion1D", 1e-9)])
def test_reference_kat_1d(oracle, name, tight):
    err, rtol = getattr(kat, name)(oracle, None)
    assert err <= rtol, f"{name}: {err:.3e} > reference rtol {rtol:.3e}"
    assert err <= tight


def test_diffusion1D_timevarying(oracle):
    err, rtol = kat.diffusion1D(oracle, None, steadyflow=False)
    assert err <= rtol and err <= 1e-9


def test_diffusion2D_timevarying(oracle):
    err, rtol = kat.diffusion2D(oracle, None, steadyflow=False)
    assert err <= rtol and err <= 1e-9


@pytest.mark.parametrize("stepper,tight", [("RK4", 1e-9), ("ETDRK4", 1e-11)])
def test_diffusion_multilayerqg(oracle, stepper, tight):
    """test/runtests.jl:50-52 runs it with stepper "RK4" (ETDRK4, exact for
    diffusion, lands at round-off).  The Filtered steppers would not pass it:
    the filter damps the Gaussian's modes above 0.65 of the Nyquist
    wavenumber, a 3.5e-6 error against the 3.3e-7 tolerance."""
    err, rtol = kat.diffusion_multilayerqg(oracle, None, stepper=stepper)
    assert err <= rtol and err <= tight


def test_clock_t_freeze_is_what_the_reference_tests_pin(oracle):
    """The reference evaluates a time-varying flow at clock.t for all stages
    (src/traceradvectiondiffusion.jl:718); test_timedependentvel2D only passes
    with that rule.  Stage-time evaluation misses its tolerance."""
    err, rtol = kat.timedependentvel2D(oracle, None)
    assert err <= rtol
    err_stage, _ = kat.timedependentvel2D(oracle, None, stage_time=True)
    assert err_stage > rtol


def test_etdrk4_exact_for_diffusion(oracle):
    """ETDRK4 integrates the linear part exactly: the heat-kernel KAT lands at
    round-off (no reference test covers ETDRK4)."""
    err, rtol = kat.diffusion2D(oracle, None, stepper="ETDRK4")
    assert err <= 1e-11
    err, rtol = kat.hyperdiffusion(oracle, None, stepper="ETDRK4")
    assert err <= 1e-11


def test_reference_kat_3d_diffusion(oracle):
    # σ=0.1 on a 64³ grid (dx≈0.098) is under-resolved: the spatial error is
    # ≈4.06e-4 whatever the stepper, which is why the reference loosens this
    # test to n³·nsteps·1e-10 = 5.2e-4.
    err, rtol = kat.diffusion3D(oracle, None)
    assert err <= rtol and err <= 4.1e-4


@pytest.mark.parametrize("name,tight", [("constvel3D", 2e-8), ("timedependentvel3D", 1e-10)])
def test_reference_kat_3d_advection(oracle, name, tight):
    err, rtol = getattr(kat, name)(oracle, None, n=128)  # the reference's 128³
    assert err <= rtol and err <= tight


def test_noflow(oracle):
    assert oracle.noflow(np.pi) == 0  # test/runtests.jl:56


def test_etdrk4_coefficients_limits(oracle):
    """φ-coefficients reduce to dt·{1/2, 1/6, 1/6, 1/6} (ζ = dt(e^{z/2}-1)/z -> dt/2) at L = 0."""
    dt = 0.01
    E, E2, z, a, b, g = oracle.etdrk4_coefficients(dt, np.array([0.0, -1e-3, -50.0]))
    assert abs(z[0] - dt / 2) < 1e-16 and abs(a[0] - dt / 6) < 1e-16
    assert abs(b[0] - dt / 6) < 1e-16 and abs(g[0] - dt / 6) < 1e-16
    # direct formula where it is well conditioned
    zz = -50.0 * dt
    assert abs(z[2] - dt * (np.exp(zz / 2) - 1) / zz) < 1e-15
    assert abs(a[2] - dt * (-4 - zz + np.exp(zz) * (4 - 3 * zz + zz * zz)) / zz ** 3) < 1e-12


def test_filter_shape(oracle):
    """FourierFlows' filter: 1 below innerK = 0.65, tol = 1e-15 at K = outerK = 1
    (the Nyquist wavenumber of a 1D grid), monotone in between."""
    g = oracle.Grid(1, 64, 2 * np.pi)
    f = oracle.makefilter(g)
    K = g.kr * g.dx / np.pi
    assert np.all(f[K < 0.65] == 1.0)
    assert abs(f[-1] - 1e-15) < 1e-17
    assert np.all(np.diff(f) <= 0)


def test_filtered_step_is_step_then_filter(oracle):
    r = oracle.Problem(oracle.TwoDAdvectingFlow(u=lambda x, y: np.sin(y), v=lambda x, y: 0 * x), nx=32,
                       kappa=1e-3, dt=0.01, stepper="RK4")
    q = oracle.Problem(oracle.TwoDAdvectingFlow(u=lambda x, y: np.sin(y), v=lambda x, y: 0 * x), nx=32,
                       kappa=1e-3, dt=0.01, stepper="FilteredRK4")
    x, y = r.grid.gridpoints()
    c0 = np.exp(-(x ** 2 + y ** 2))
    oracle.set_c(r, c0)
    oracle.set_c(q, c0)
    oracle.stepforward(r, 1)
    oracle.stepforward(q, 1)
    assert np.allclose(q.sol, r.sol * oracle.makefilter(r.grid), rtol=0, atol=1e-14)
