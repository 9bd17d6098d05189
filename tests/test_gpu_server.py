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


def test_served_fp32_mean_and_mass_drift_vs_oracle(gpu, oracle):
    """A served FP32 request keeps its (0,0) mode in FP64: the result's mean
    matches the FP64 oracle to 1e-9 relative, and the server's per-request
    mass record (sum of c0, sum of the result) gives the same drift as the
    oracle's."""
    from test_gpu_batched import _uniform_damping_case
    spec, c0, u, v, r = _uniform_damping_case(gpu, oracle, n=128, nsteps=200)
    s = gpu.Server(T=np.float32, chunk_steps=30)
    rid = s.submit(spec, c0, u, v)
    s.wait_all(300)
    state, c = s.poll(rid)
    assert state == "done"
    assert abs(c.sum() - r.vars.c.sum()) <= 1e-9 * abs(r.vars.c.sum())
    assert oracle.rel_l2(c, r.vars.c) <= 1e-5
    info = s.result_info(rid)
    drift_oracle = r.vars.c.sum() / c0.sum() - 1
    assert abs(info["mass0"] - c0.sum()) <= 1e-12 * abs(c0.sum())
    assert abs(info["mass_drift"] - drift_oracle) <= 1e-9
    assert s.stats()["mass_drift_max_abs"] == pytest.approx(abs(info["mass_drift"]), rel=1e-12)
    s.close()


def test_over_budget_request_refused_at_submit(gpu):
    """A request that could not fit even in an empty server is refused at
    submission with PTF_ERR_MEMORY instead of queueing for ever; one that
    fits is still served."""
    s = gpu.Server(T=np.float32, memory_budget=32 << 20, slots_per_bucket=1)
    u, v = cellular_arrays(1024)
    with pytest.raises(MemoryError):
        s.submit(gpu.SolveSpec(n=1024, nsteps=2, dt=1e-3, kappa=1e-3), gauss(1024, 0, 0, 0.4), u, v)
    st = s.stats()
    assert st["queued"] == 0 and st["active"] == 0
    n = 64
    u, v = cellular_arrays(n)
    rid = s.submit(gpu.SolveSpec(n=n, nsteps=4, dt=1e-3, kappa=1e-3), gauss(n, 0, 0, 0.4), u, v)
    s.wait_all(120)
    assert s.poll(rid)[0] == "done"
    s.close()


def test_budget_reclaims_empty_buckets(gpu):
    """Under a tight budget, a bucket of one size whose solves all finished is
    released so that a request of another size can be admitted."""
    # 20 MiB: the server's fixed buffers (about 9 MB) and a two-slot 256^2
    # bucket (4.9 MB) leave no room for a 512^2 slot (9.6 MB) until the 256^2
    # bucket is empty and released
    budget = 20 << 20
    s = gpu.Server(T=np.float32, memory_budget=budget, slots_per_bucket=2, chunk_steps=5)
    ids = []
    for n in (256, 512, 256):
        u, v = cellular_arrays(n)
        ids.append(s.submit(gpu.SolveSpec(n=n, nsteps=6, dt=1e-3, kappa=1e-3), gauss(n, 0, 0, 0.4), u, v))
    s.wait_all(300)
    assert [s.poll(i)[0] for i in ids] == ["done"] * 3
    assert s.stats()["device_bytes"] <= budget
    s.close()


def _state(s, rid):
    try:
        return s.poll(rid)[0]
    except Exception:
        return "failed"


def _wait_states(s, ids, timeout):
    t0 = time.time()
    while time.time() - t0 < timeout:
        if all(_state(s, i) in ("done", "failed") for i in ids):
            return
        time.sleep(0.01)
    raise TimeoutError("requests did not finish")


def test_injected_step_failure_releases_slots_and_handles(gpu):
    """A chunk that fails (injected on the host: nothing faults on the GPU)
    fails the requests in flight and releases their batch slots and 3D
    handles; the server keeps serving new requests in the freed slots."""
    s = gpu.Server(T=np.float32, chunk_steps=3, slots_per_bucket=4)
    n = 64
    u, v = cellular_arrays(n)
    x = -np.pi + 2 * np.pi / 16 * np.arange(16)
    Z, Y, X = np.meshgrid(x, x, x, indexing="ij")
    s.inject_step_failure(0)
    doomed = [s.submit(gpu.SolveSpec(n=n, nsteps=50, dt=1e-3, kappa=1e-3), gauss(n, 0.1 * i, 0, 0.4), u, v)
              for i in range(3)]
    doomed.append(s.submit(gpu.SolveSpec(n=16, dim=3, nsteps=50, dt=1e-3, kappa=1e-3),
                           np.exp(-(X ** 2 + Y ** 2 + Z ** 2)), np.cos(Y), np.cos(Z), np.cos(X)))
    with pytest.raises(Exception):
        s.wait_all(120)
    st = s.stats()
    assert st["failed"] >= 1 and st["active"] == 0
    assert st["batch_solves"] == 0 and st["handles"] == 0
    states = [_state(s, rid) for rid in doomed]
    assert "failed" in states and set(states) <= {"failed", "done"}
    ok = [s.submit(gpu.SolveSpec(n=n, nsteps=5, dt=1e-3, kappa=1e-3), gauss(n, 0, 0.2 * i, 0.4), u, v)
          for i in range(4)]
    _wait_states(s, ok, 120)
    assert all(s.poll(i)[0] == "done" for i in ok)
    assert s.stats()["batch_solves"] == 0
    s.close()
