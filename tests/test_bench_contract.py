"""`bench.py --impl reference` (the FP64 oracle timed on the host cores) on
the CPU: one JSON line with the keys of the result contract, and nothing
from ranks other than 0 under a multi-process launch."""
import json
import os
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent

KEYS = {"impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
        "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"}


def _run(extra_env=None, *args):
    env = dict(os.environ)
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        env.pop(k, None)
    env.update(extra_env or {})
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", *args],
                       capture_output=True, text=True, env=env, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    return [ln for ln in r.stdout.splitlines() if ln.strip()]


def test_reference_arm_line():
    lines = _run(None, "--n", "128", "--steps", "4", "--warmup", "3")
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert KEYS <= set(d)
    assert d["impl"] == "reference" and d["n_gpus"] == 1 and d["steps"] == 4 and d["warmup"] == 3
    assert d["value"] > 0 and d["higher_is_better"] is True and d["scaling"] == "weak"
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["cpu_baseline"]["value"] == d["value"] == d["e2e"]["value"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["config"]["nx"] == 128 and d["config"]["workload"]


def test_reference_arm_other_ranks_are_silent():
    assert _run({"WORLD_SIZE": "2", "RANK": "1", "LOCAL_RANK": "1"}, "--n", "64", "--steps", "1") == []


def _bench():
    import importlib.util
    spec = importlib.util.spec_from_file_location("ptf_bench_mod", ROOT / "bench.py")
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def test_served_stream_flows_follow_the_workload_definition():
    """The served stream's random-phase flows: incompressible, rms speed 1,
    energy only in 4 <= |k| <= 16 with |u_k| ~ |k|^-3 (2D streamfunction; 3D
    curl of a vector potential)."""
    import numpy as np
    b = _bench()
    rng = np.random.default_rng(0)
    n = 64
    u, v = b.random_phase_flow(n, rng)
    assert abs(np.sqrt(np.mean(u ** 2 + v ** 2)) - 1) < 1e-12
    uh, vh = np.fft.rfft2(u), np.fft.rfft2(v)
    l = np.fft.fftfreq(n, 1.0 / n)[:, None]
    k = np.arange(n // 2 + 1)[None, :]
    div = k * uh + l * vh
    assert np.abs(div).max() <= 1e-10 * np.abs(uh).max()
    K = np.sqrt(k ** 2 + l ** 2)
    e = np.abs(uh) ** 2 + np.abs(vh) ** 2
    assert e[(K < 4) | (K > 16)].max() <= 1e-20 * e.max()
    # |u_k| |k|^3 is the same for every mode of the band (random phases only)
    band = (K >= 4) & (K <= 16) & (k > 0) & (k < n // 2)
    r = np.sqrt(e[band]) * K[band] ** 3
    assert r.max() / r.min() < 1 + 1e-9
    u3, v3, w3 = b.random_phase_flow(32, rng, dim=3)
    assert abs(np.sqrt(np.mean(u3 ** 2 + v3 ** 2 + w3 ** 2)) - 1) < 1e-12
    m3 = np.fft.fftfreq(32, 1.0 / 32)[:, None, None]
    l3 = np.fft.fftfreq(32, 1.0 / 32)[None, :, None]
    k3 = np.arange(17)[None, None, :]
    div3 = k3 * np.fft.rfftn(u3) + l3 * np.fft.rfftn(v3) + m3 * np.fft.rfftn(w3)
    assert np.abs(div3).max() <= 1e-10 * np.abs(np.fft.rfftn(u3)).max()


def test_clock_summary_reports_throttle_reasons():
    """The `clocks` object: median SM clock under load and every throttle
    reason seen Active (a run with a slowdown reason is re-measured)."""
    b = _bench()
    rows = ["0, 2070, 2070, 900.1, 0x0, Not Active, Not Active, Not Active, Not Active",
            "0, 2055, 2070, 1350.0, 0x4, Not Active, Not Active, Not Active, Active",
            "0, 1900, 2070, 1400.0, 0x8, Active, Not Active, Not Active, Active",
            "", "0, [N/A], 2070, 0, 0x0, , , , "]
    c = b.ClockSampler.summarize(rows)
    assert c["samples"] == 3 and c["sm_mhz"] == 2055.0 and c["sm_max_mhz"] == 2070.0
    assert c["reasons"] == ["hw_slowdown", "sw_power_cap"]
    assert b.ClockSampler.summarize([]) == {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}


def test_roofline_traffic_comes_from_the_committed_profile():
    """`roofline.traffic` of the default run is the ncu DRAM bytes per launch
    recorded in profiles/, for the dominant pass of that workload."""
    b = _bench()
    col, src = b.profiled_traffic("column_pass", "f32", 1024, 16)
    row, _ = b.profiled_traffic("row_pass", "f32", 1024, 16)
    assert src == "pass2d_fp32_1024x1024_b16_etdrk4.md"
    assert col == 399764672 and row == 183517504
    assert b.profiled_traffic("column_pass", "f32", 2048, 16) == (None, None)
    peak, kind = b.load_peaks()
    assert peak > 1000 and kind in ("measured", "fallback")


def test_fp64_pipe_activity_comes_from_the_committed_profile():
    """`fp64_plain.roofline` carries the FP64-pipe activity ncu measured in
    the same passes, read from profiles/."""
    b = _bench()
    col, src = b.profiled_fp64_pipe("column_pass", 1024)
    row, _ = b.profiled_fp64_pipe("row_pass", 1024)
    assert src == "pass2d_fp64_1024x1024_b1_etdrk4.md"
    assert col == 69.0 and row == 68.4
    assert b.profiled_fp64_pipe("column_pass", 4096) == (None, None)
