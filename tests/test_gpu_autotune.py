"""Launch-shape tuning: ptf_autotune / ptf_set_tuning change the time per step
only.  The solve is left where it was, and steps after tuning agree with an
untuned problem (the per-line arithmetic does not depend on the shapes)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def cellular():
    return (lambda x, y: np.cos(x) * np.sin(y), lambda x, y: -np.sin(x) * np.cos(y))


def make(gpu, n, T, batch=1, stepper="ETDRK4"):
    u, v = cellular()
    return gpu.Problem(gpu.GPU(), gpu.TwoDAdvectingFlow(u=u, v=v), nx=n, κ=1e-3, dt=0.001, stepper=stepper, T=T,
                       batch=batch)


def ic(gpu, p, batch=1):
    x, y = gpu.gridpoints(p.grid)
    c = np.exp(-((x - 2.0) ** 2 + (y - 3.0) ** 2) / 0.3)
    return np.stack([c * (b + 1) for b in range(batch)]) if batch > 1 else c


@pytest.mark.parametrize("n,T,batch,tol", [(256, np.float64, 1, 1e-13), (512, np.float32, 4, 2e-6)])
def test_autotune_keeps_state_and_results(gpu, oracle, n, T, batch, tol):
    p = make(gpu, n, T, batch)
    q = make(gpu, n, T, batch)
    c0 = ic(gpu, p, batch)
    gpu.set_c(p, c0)
    gpu.set_c(q, c0)
    gpu.stepforward(p, 3)
    gpu.stepforward(q, 3)
    before = p.sol
    t = p.autotune(trial_steps=2, force=True)
    assert t["ms_per_step"] > 0
    assert np.array_equal(p.sol, before)
    assert p.clock.step == 3
    gpu.stepforward(p, 5)
    gpu.stepforward(q, 5)
    gpu.updatevars(p)
    gpu.updatevars(q)
    assert oracle.rel_l2(p.vars.c, q.vars.c) <= tol
    # cached: a second problem of the same shape takes the same shapes
    r = make(gpu, n, T, batch)
    gpu.set_c(r, c0)
    t2 = r.autotune(trial_steps=2)
    assert {k: t2[k] for k in t2 if k != "ms_per_step"} == {k: t[k] for k in t if k != "ms_per_step"}


def test_set_tuning_validates(gpu):
    p = make(gpu, 128, np.float32)
    t = p.tuning
    assert t["col_lines"] >= 1 and t["row_pairs"] >= 1
    with pytest.raises(Exception):
        p.tuning = {"col_lines": 3}
    with pytest.raises(Exception):
        p.tuning = {"row_pairs": 4096}
    with pytest.raises(Exception):
        p.tuning = {"branches": 9}
    assert p.tuning == t


@pytest.mark.parametrize("shape", [dict(col_lines=1, row_pairs=1), dict(col_lines=2, row_pairs=2, row_staged=1),
                                   dict(branches=2, solves_per_group=1)])
def test_every_shape_same_result(gpu, oracle, shape):
    p = make(gpu, 256, np.float64, batch=2)
    q = make(gpu, 256, np.float64, batch=2)
    p.tuning = shape
    c0 = ic(gpu, p, 2)
    gpu.set_c(p, c0)
    gpu.set_c(q, c0)
    gpu.stepforward(p, 4)
    gpu.stepforward(q, 4)
    gpu.updatevars(p)
    gpu.updatevars(q)
    assert oracle.rel_l2(p.vars.c, q.vars.c) <= 1e-13
