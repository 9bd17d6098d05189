"""Generate the golden fixtures in this directory from the CPU oracle.

The reference (Julia + FourierFlows) cannot run in this environment, so the
fixtures are produced by the FP64 oracle (oracle/ptf_oracle.py), which is
itself pinned to the reference's known-answer tests (tests/test_oracle_kat.py).
They freeze the oracle's output on the benchmark workloads so that GPU runs
can be checked without re-running long CPU solves, and so that any change of
the oracle shows up as a fixture mismatch.

Run:  python tests/golden/make_golden.py
"""
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent / "oracle"))
import ptf_oracle as o  # noqa: E402


def cellular_flow(U=1.0, k=1.0):
    """ψ = U cos(kx) cos(ky); u = -∂ψ/∂y, v = ∂ψ/∂x (examples/cellularflow.jl:57-58 signs)."""
    u = lambda x, y: U * k * np.cos(k * x) * np.sin(k * y)
    v = lambda x, y: -U * k * np.sin(k * x) * np.cos(k * y)
    return u, v


def gaussian(x, y, x0, y0, s):
    return np.exp(-((x - x0) ** 2 + (y - y0) ** 2) / (2 * s ** 2))


def cellular128_rk4():
    """Cellular flow, 128², κ=0.002, η=0, RK4, dt=0.01; c at steps 100 and 2000."""
    u, v = cellular_flow()
    p = o.Problem(o.TwoDAdvectingFlow(u=u, v=v), nx=128, Lx=2 * np.pi, kappa=0.002, eta=0.0, dt=0.01, stepper="RK4")
    x, y = p.grid.gridpoints()
    c0 = gaussian(x, y, np.pi / 2, np.pi / 2, 0.2)
    o.set_c(p, c0)
    o.stepforward(p, 100); o.updatevars(p)
    c100 = p.vars.c.copy()
    o.stepforward(p, 1900); o.updatevars(p)
    return dict(c0=c0, c100=c100, c2000=p.vars.c.copy(), t=p.clock.t, step=p.clock.step)


def cellular128_etdrk4():
    """Cellular flow k=4, U=1, κ=η=1e-4, κh=1e-12, nκh=2, ETDRK4, dt=0.002, 128²; c at step 50.

    t = 0.1 keeps the tracer resolved: the flow's strain (≈16) thins the
    filaments like e^{-16 t}, and without dealiasing the run becomes
    aliasing-unstable near t ≈ 0.3 at 128² and 256²."""
    u, v = cellular_flow(1.0, 4.0)
    p = o.Problem(o.TwoDAdvectingFlow(u=u, v=v), nx=128, Lx=2 * np.pi, kappa=1e-4, eta=1e-4, kappah=1e-12,
                  nkappah=2, dt=0.002, stepper="ETDRK4")
    x, y = p.grid.gridpoints()
    c0 = gaussian(x, y, np.pi / 2, np.pi / 2, 0.2)
    o.set_c(p, c0)
    o.stepforward(p, 50); o.updatevars(p)
    return dict(c50=p.vars.c.copy(), t=p.clock.t, step=p.clock.step)


def abc_flow(A=1.0, B=np.sqrt(2 / 3), C=np.sqrt(1 / 3)):
    """ABC flow: u = A sin z + C cos y, v = B sin x + A cos z, w = C sin y + B cos x."""
    u = lambda x, y, z: A * np.sin(z) + C * np.cos(y)
    v = lambda x, y, z: B * np.sin(x) + A * np.cos(z)
    w = lambda x, y, z: C * np.sin(y) + B * np.cos(x)
    return u, v, w


def abc32_etdrk4():
    """3D ABC flow, 32³, κ=η=ι=5e-4, Gaussian σ=0.3 at the domain centre, ETDRK4, dt=0.005; c at step 100."""
    u, v, w = abc_flow()
    p = o.Problem(o.ThreeDAdvectingFlow(u=u, v=v, w=w), nx=32, Lx=2 * np.pi, kappa=5e-4, dt=0.005, stepper="ETDRK4")
    x, y, z = p.grid.gridpoints()
    c0 = np.exp(-(x ** 2 + y ** 2 + z ** 2) / (2 * 0.3 ** 2))
    o.set_c(p, c0)
    o.stepforward(p, 100); o.updatevars(p)
    return dict(c0=c0, c100=p.vars.c.copy(), t=p.clock.t, step=p.clock.step)


def line256():
    """1D, 256 points, u = 0.4 + 0.2 cos x, κ=1e-3, a Gaussian σ=0.3 plus a
    cos 3x ripple; RK4 and ETDRK4, dt=0.005, c at step 400 (t = 2)."""
    out = {}
    for stepper in ("RK4", "ETDRK4"):
        p = o.Problem(o.OneDAdvectingFlow(u=lambda x: 0.4 + 0.2 * np.cos(x)), nx=256, Lx=2 * np.pi, kappa=1e-3,
                      dt=0.005, stepper=stepper)
        (x,) = p.grid.gridpoints()
        c0 = np.exp(-x ** 2 / (2 * 0.3 ** 2)) + 0.1 * np.cos(3 * x)
        o.set_c(p, c0)
        o.stepforward(p, 400); o.updatevars(p)
        out["c0"] = c0
        out[f"c400_{stepper}"] = p.vars.c.copy()
        out["t"], out["step"] = p.clock.t, p.clock.step
    return out


FIXTURES = {"cellular128_rk4": cellular128_rk4, "cellular128_etdrk4": cellular128_etdrk4,
            "abc32_etdrk4": abc32_etdrk4, "line256": line256}

if __name__ == "__main__":
    names = sys.argv[1:] or list(FIXTURES)
    for name in names:
        d = FIXTURES[name]()
        np.savez_compressed(HERE / f"{name}.npz", **d)
        print("wrote", name)
