"""Snapshot output (FourierFlows Output / saveproblem / saveoutput, as the
reference's examples use them, examples/onedim_gaussiandiffusion.jl:74-88):
the JLD2 group layout written to an appendable .npz, on a host stand-in of a
problem (no device needed)."""
import types

import numpy as np
import pytest


def _stub(pkg, dim=2, n=16):
    grid = pkg.TracerAdvectionDiffusion._Grid(dim, n, 2 * np.pi)
    cfg = types.SimpleNamespace(kappa=1e-3, eta=2e-3, iota=3e-3, kappah=1e-9, nkappah=2, dt=0.01)
    clock = types.SimpleNamespace(step=0, t=0.0)
    prob = types.SimpleNamespace(grid=grid, _cfg=cfg, clock=clock,
                                 vars=types.SimpleNamespace(c=np.zeros(grid.shape)),
                                 sol=np.zeros(grid.spec_shape, complex))
    return prob


def test_output_layout_and_append(pkg, tmp_path):
    prob = _stub(pkg)
    field = lambda p: np.full(p.grid.shape, float(p.clock.step))
    out = pkg.Output(prob, tmp_path / "run.jld2", ("concentration", field))
    pkg.saveproblem(out)
    for step in range(0, 151, 50):
        prob.clock.step, prob.clock.t = step, 0.01 * step
        pkg.saveoutput(out)
    f = pkg.jldopen(out.path)
    assert f.keys() == ["clock", "eqn", "grid", "params", "snapshots"]
    steps = sorted(int(k) for k in f["snapshots/t"].keys())
    assert steps == [0, 50, 100, 150]
    assert [f[f"snapshots/t/{i}"] for i in steps] == [0.0, 0.5, 1.0, 1.5]
    for i in steps:
        assert np.array_equal(f[f"snapshots/concentration/{i}"], np.full((16, 16), float(i)))
    assert f["grid/Lx"] == 2 * np.pi and np.array_equal(f["grid/x"], prob.grid.x)
    assert f["params/κ"] == 1e-3 and f["params/η"] == 2e-3 and f["clock/dt"] == 0.01
    L = f["eqn/L"]
    K2 = prob.grid.Krsq
    assert L.shape == prob.grid.spec_shape
    assert np.allclose(L, -1e-3 * prob.grid.kr[None, :] ** 2 - 2e-3 * prob.grid.l[:, None] ** 2 - 1e-9 * K2 ** 2)
    f.close()
    # plain numpy reads the same members
    with np.load(out.path) as z:
        assert float(z["snapshots/t/100"]) == 1.0


def test_output_never_overwrites(pkg, tmp_path):
    prob = _stub(pkg, dim=1)
    a = pkg.Output(prob, tmp_path / "x.jld2")
    b = pkg.Output(prob, tmp_path / "x.jld2")
    assert a.path.name == "x.jld2" and b.path.name == "x_1.jld2"
    pkg.saveoutput(a)
    with pytest.raises(ValueError):
        pkg.saveoutput(a)  # same step twice
    with pytest.raises(TypeError):
        pkg.Output(prob, tmp_path / "y.jld2", ("c",))
