"""Request server (ptf_server_*): continuous batching with admission by
memory budget; every result is the same alone and in the mix."""
import time

import numpy as np
import pytest

from test_gpu_batched import cellular_arrays, gauss

pytestmark = pytest.mark.gpu


def run_alone(gpu, spec, c0, u, v, T):
    s = gpu.Server(T=T)
    rid = s.submit(spec, c0, u, v)
    s.wait_all(120)
    state, c = s.poll(rid)
    s.close()
    assert state == "done"
    return c


@pytest.mark.parametrize("T", [np.float64, np.float32])
def test_result_alone_equals_result_in_mix(gpu, T):
    rng = np.random.default_rng(3)
    target = gpu.SolveSpec(n=128, nsteps=30, dt=0.004, kappa=2e-3)
    u, v = cellular_arrays(128)
    c0 = gauss(128, 0.4, -0.3, 0.5)
    alone = run_alone(gpu, target, c0, u, v, T)
    s = gpu.Server(T=T, chunk_steps=7)
    ids = []
    for i in range(12):
        n = int(rng.choice([64, 128, 256]))
        uu, vv = cellular_arrays(n, k=1 + i % 3)
        spec = gpu.SolveSpec(n=n, nsteps=int(rng.integers(5, 60)), dt=0.003, kappa=float(10 ** rng.uniform(-4, -2)))
        ids.append(s.submit(spec, gauss(n, *rng.uniform(-2, 2, 2), 0.4), uu, vv))
        if i == 5:
            mine = s.submit(target, c0, u, v)  # arrives while others are on the GPU
        time.sleep(0.002)
    s.wait_all(300)
    state, c = s.poll(mine)
    assert state == "done"
    # identical arithmetic alone and in the mix: bit-identical in practice; the stated tolerance is 1e-12 (FP64)
    err = np.linalg.norm(c - alone) / np.linalg.norm(alone)
    assert err <= (1e-12 if T == np.float64 else 1e-6)
    st = s.stats()
    assert st["completed"] == 13 and st["failed"] == 0
    assert 0 < st["p50_s"] <= st["p99_s"]
    s.close()


def test_admission_by_memory_budget(gpu):
    """A budget that holds a few solves at a time still completes all requests
    (they queue and are admitted as memory frees up)."""
    n = 256
    u, v = cellular_arrays(n)
    s = gpu.Server(T=np.float32, memory_budget=24 << 20, slots_per_bucket=2, chunk_steps=5)
    ids = [s.submit(gpu.SolveSpec(n=n, nsteps=10, dt=0.002, kappa=1e-3), gauss(n, 0.1 * i, 0, 0.4), u, v)
           for i in range(10)]
    s.wait_all(300)
    st = s.stats()
    assert st["completed"] == 10 and st["device_bytes"] <= 24 << 20
    for rid in ids:
        assert s.poll(rid)[0] == "done"
    s.close()


def test_server_3d_request(gpu, oracle):
    n = 32
    x = -np.pi + 2 * np.pi / n * np.arange(n)
    Z, Y, X = np.meshgrid(x, x, x, indexing="ij")
    A, B, C = 1.0, np.sqrt(2 / 3), np.sqrt(1 / 3)
    u = A * np.sin(Z) + C * np.cos(Y)
    v = B * np.sin(X) + A * np.cos(Z)
    w = C * np.sin(Y) + B * np.cos(X)
    c0 = np.exp(-(X ** 2 + Y ** 2 + Z ** 2) / (2 * 0.4 ** 2))
    s = gpu.Server(T=np.float64)
    rid = s.submit(gpu.SolveSpec(n=n, dim=3, nsteps=6, dt=0.01, kappa=1e-3), c0, u, v, w)
    s.wait_all(120)
    state, c = s.poll(rid)
    assert state == "done"
    r = oracle.Problem(oracle.ThreeDAdvectingFlow(u=lambda *a: u, v=lambda *a: v, w=lambda *a: w), nx=n,
                       kappa=1e-3, dt=0.01)
    oracle.set_c(r, c0)
    oracle.stepforward(r, 6)
    oracle.updatevars(r)
    assert oracle.rel_l2(c, r.vars.c) <= 1e-12
    s.close()
