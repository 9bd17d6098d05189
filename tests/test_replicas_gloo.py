"""Multi-GPU form: replicas only.  `bench.py --gpus N` runs one process per
GPU, each stepping its own batch of independent solves from its own seed; the
only collectives are the barrier around the timed region and the max of the
ranks' times, and the job's rate is all ranks' units over the slowest rank's
time.  Checked here with two `gloo` ranks on the CPU (no GPU involved)."""
import importlib.util
import json
import os
import socket
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def _bench():
    spec = importlib.util.spec_from_file_location("ptf_bench", ROOT / "bench.py")
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    b = _bench()
    b.init_ranks("gloo")
    w, r, local = b.dist_setup()
    seed = b.replica_seed(r)
    c0 = b.initial_conditions(32, 2, seed)
    my_seconds = 1.0 + 0.5 * r  # rank 1 is the slow one
    dist.barrier()
    slowest = b.max_over_ranks(my_seconds, w, "cpu")
    rate = b.job_rate(w, 2 * 32 * 32 * 10, slowest)
    dist.barrier()
    Path(out_dir, f"rank{r}.json").write_text(json.dumps(
        {"world": w, "rank": r, "local": local, "seed": seed, "checksum": float(c0.sum()),
         "first": float(c0[0, 0, 0]), "slowest": slowest, "rate": rate}))
    dist.destroy_process_group()


def test_two_gloo_replicas(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, start_method="spawn", join=True)
    res = [json.loads((tmp_path / f"rank{r}.json").read_text()) for r in range(2)]
    assert [x["rank"] for x in res] == [0, 1] and all(x["world"] == 2 for x in res)
    # independent work: different seeds give different initial conditions
    assert res[0]["seed"] != res[1]["seed"]
    assert res[0]["checksum"] != res[1]["checksum"]
    # every rank sees the slowest rank's time, and the job rate uses it
    assert all(x["slowest"] == 1.5 for x in res)
    assert all(abs(x["rate"] - 2 * 2 * 32 * 32 * 10 / 1.5) < 1e-6 for x in res)


def _rank_fails(rank, world, port, out_dir, mode):
    import time
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    b = _bench()
    b.init_ranks("gloo", timeout_s=5)
    if rank == 1:
        if mode == "stalls":  # alive but never reaches the barrier (until rank 0 has given up)
            t_end = time.monotonic() + 60
            while not Path(out_dir, "rank0.json").exists() and time.monotonic() < t_end:
                time.sleep(0.1)
        return  # "leaves": exits between steps without reaching the barrier
    t0 = time.monotonic()
    try:
        dist.barrier()
        outcome = "returned"
    except Exception as e:  # the backend's error for a peer that is gone or late
        outcome = type(e).__name__
    Path(out_dir, "rank0.json").write_text(json.dumps({"outcome": outcome, "seconds": time.monotonic() - t0}))


@pytest.mark.parametrize("mode", ["leaves", "stalls"])
def test_a_failed_rank_ends_the_next_collective_with_an_error(tmp_path, mode):
    """Failure detection on the host: rank 1 exits, or stays alive without
    reaching the barrier; rank 0's barrier fails with an error (at once for a
    rank that is gone, after the 5 s process-group timeout for one that
    stalls) instead of waiting for ever."""
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    mp.start_processes(_rank_fails, args=(2, _free_port(), str(tmp_path), mode), nprocs=2, start_method="spawn",
                       join=True)
    r = json.loads((tmp_path / "rank0.json").read_text())
    assert r["outcome"] != "returned"
    assert r["seconds"] < 30


def test_single_process_defaults():
    b = _bench()
    env = {k: os.environ.pop(k) for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK") if k in os.environ}
    try:
        assert b.dist_setup() == (1, 0, 0)
        assert b.max_over_ranks(3.0, 1, "cpu") == 3.0
        assert b.job_rate(1, 100, 2.0) == 50.0
    finally:
        os.environ.update(env)
    c = b.initial_conditions(16, 3, b.replica_seed(0))
    assert c.shape == (3, 16, 16) and np.isfinite(c).all()
