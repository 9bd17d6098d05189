"""Failure detection on the GPU without a fault: a bounded wait in a kernel
runs out on purpose and the host reads the error status, with the CUDA
context still usable.

The persistent batched stage kernel makes a column item wait until its
bucket's row items are done (a device counter, a bounded spin with
``__nanosleep``).  ``inject_wait_timeout`` makes the column items wait for one
row item more than exists -- a count nothing reaches -- with a short limit,
so the wait gives up, the item is skipped, the kernel ends, and
``synchronize`` reports ``PTF_ERR_CUDA``.  Nothing traps, faults or waits
without a bound; a fresh batch afterwards steps correctly.
"""
import time

import numpy as np
import pytest

from test_gpu_batched import cellular_arrays, gauss

pytestmark = pytest.mark.gpu


def _case(gpu, n=64, nsteps=6):
    u, v = cellular_arrays(n)
    spec = gpu.SolveSpec(n=n, nsteps=nsteps, dt=0.004, kappa=2e-3)
    return spec, gauss(n, 0.3, -0.2, 0.5), u, v


def test_bounded_wait_runs_out_and_is_reported(gpu):
    from ptf_gb300._lib import PtfError
    spec, c0, u, v = _case(gpu)
    b = gpu.BatchedProblem(T=np.float32, persistent=True, slots_per_bucket=1)
    b.add(spec, c0, u, v)
    b.step(1)
    b.synchronize()  # the normal wait: fine
    # about 2^22 sleeps of ~128 ns (~0.5 s) per wait; one column item per stage
    b.inject_wait_timeout(extra_row_items=1, spin_limit=1 << 22)
    t0 = time.time()
    b.step(1)
    with pytest.raises(PtfError, match="gave up waiting"):
        b.synchronize()
    assert time.time() - t0 < 60
    b.close()


def test_context_usable_after_wait_timeout(gpu, oracle):
    """After a run-out wait, a fresh batch (persistent and two-launch forms)
    and a single-solve handle still give the right answer."""
    spec, c0, u, v = _case(gpu)
    bad = gpu.BatchedProblem(T=np.float64, persistent=True, slots_per_bucket=1)
    bad.add(spec, c0, u, v)
    bad.inject_wait_timeout(extra_row_items=3, spin_limit=1 << 21)
    bad.step(2)
    with pytest.raises(Exception):
        bad.synchronize()
    bad.close()
    r = oracle.Problem(oracle.TwoDAdvectingFlow(u=lambda *a: u, v=lambda *a: v), nx=spec.n, kappa=spec.kappa,
                       dt=spec.dt)
    oracle.set_c(r, c0)
    oracle.stepforward(r, spec.nsteps)
    oracle.updatevars(r)
    for persistent in (True, False):
        b = gpu.BatchedProblem(T=np.float64, persistent=persistent, slots_per_bucket=2)
        sid = b.add(spec, c0, u, v)
        b.step(spec.nsteps)
        b.synchronize()
        assert oracle.rel_l2(b.get_c(sid), r.vars.c) <= 1e-12
        b.close()
    p = gpu.Problem(gpu.GPU(), gpu.TwoDAdvectingFlow(), nx=spec.n, κ=spec.kappa, η=spec.kappa, dt=spec.dt)
    p.set_flow_arrays(u, v)
    gpu.set_c(p, c0)
    gpu.stepforward(p, spec.nsteps)
    gpu.updatevars(p)
    assert oracle.rel_l2(p.vars.c, r.vars.c) <= 1e-12


def test_wait_hook_rejected_outside_persistent_form(gpu):
    from ptf_gb300._lib import PtfError
    b = gpu.BatchedProblem(T=np.float32, persistent=False)
    with pytest.raises(PtfError):
        b.inject_wait_timeout(1, 1000)
    b.close()
