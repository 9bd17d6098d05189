#!/usr/bin/env python
"""Benchmark of the TracerAdvectionDiffusion time step on GB300.

Workload (the 2D cellular-flow configuration the headline metric is quoted
on): ψ = U cos(kx) cos(ky) with k = 4, U = 1 (u = -∂ψ/∂y, v = ∂ψ/∂x), Lx = Ly =
2π, nx = ny = 1024, κ = η = 1e-4, hyperdiffusion κh = 1e-12 on ∇⁴ (nκh = 2),
ETDRK4.  Initial conditions are Gaussians of σ = 0.2 at seeded random centres
(synthetic data).

* ``value``: the FP32-batched form -- ``--batch`` independent solves (an
  ensemble of initial conditions) stepped together, FP32 bulk transforms with
  FP64 ETDRK4 coefficients.  Unit: grid-point-steps/s = batch·nx·ny·steps/s.
  The batch state (≈30 MB per solve) is larger than L2, so consecutive steps
  are timed back to back.
* ``fp64_plain``: one FP64 solve of the same workload (the drop-in path),
  each timed step preceded by an L2 flush.
* ``dt`` defaults to 5e-4: the workload's nominal dt = 2e-3 gives an advective
  CFL number u_max·k_max·dt = 4·512·2e-3 ≈ 4.1 at 1024², beyond the
  ETDRK4/RK4 stability limit (≈2.8); the FP64 CPU oracle itself diverges after
  ≈22 steps there.  The cost of a step does not depend on dt.

``--impl reference`` times the CPU FP64 oracle restatement of the reference
(NumPy + pocketfft on all host cores): the reference's own Julia code cannot
run on these machines (no Julia).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "grid-pt-steps/s (FP32-batched, rel-L2<=1e-5 vs FP64 oracle; FP64 plain beside)"
UNIT = "grid-pt-steps/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=1024)
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--dt", type=float, default=5e-4)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-oracle-check", action="store_true")
    ap.add_argument("--only-main", action="store_true", help="skip the 3D, ensemble and serving measurements")
    ap.add_argument("--serve-requests", type=int, default=600)
    ap.add_argument("--serve-requests-fp64", type=int, default=48)
    ap.add_argument("--serve-rate", type=float, default=12.0, help="Poisson arrival rate (requests/s)")
    ap.add_argument("--ensemble-steps", type=int, default=1000)
    ap.add_argument("--config-steps-2d", type=int, default=1000, help="steps of the 4096^2 configuration")
    ap.add_argument("--config-steps-3d", type=int, default=500, help="steps of the 256^3 configuration")
    ap.add_argument("--only", default="", help="comma-separated workload keys to run (default: all)")
    ap.add_argument("--workloads-only", action="store_true",
                    help="run only the secondary configurations (no contract line)")
    ap.add_argument("--no-tune", action="store_true", help="keep the default launch shapes (no ptf_autotune)")
    ap.add_argument("--acc-time", type=float, default=0.5,
                    help="simulated time of the accuracy window (0.5 = the configured 1000 steps at dt 5e-4)")
    ap.add_argument("--no-comparator", action="store_true", help="skip the torch/cuFFT comparator")
    ap.add_argument("--profile-case", action="store_true",
                    help="only step the batched workload (for ncu); prints no result line")
    ap.add_argument("--profile-fp64", action="store_true", help="with --profile-case: FP64 instead of FP32")
    return ap.parse_args()


def workload(args, batch):
    return {
        "workload": f"2D cellular flow {args.n}x{args.n}, ETDRK4, psi=U cos(4x)cos(4y) U=1, kappa=eta=1e-4, "
                    f"kappah=1e-12 nkappah=2, dt={args.dt:g}",
        "nx": args.n, "ny": args.n, "stepper": "ETDRK4", "dt": args.dt, "nominal_dt": 0.002,
        "batch_per_gpu": batch, "precision": "FP32 bulk, FP64 ETDRK4 coefficients",
        "l2_policy": "batch state larger than L2 (FP32 batched); L2 flushed before every timed step (FP64 plain)",
    }


def flow_fns():
    u = lambda x, y: 4.0 * np.cos(4 * x) * np.sin(4 * y)
    v = lambda x, y: -4.0 * np.sin(4 * x) * np.cos(4 * y)
    return u, v


def initial_conditions(n, batch, seed):
    rng = np.random.default_rng(seed)
    x = -np.pi + 2 * np.pi / n * np.arange(n)
    Y, X = np.meshgrid(x, x, indexing="ij")
    out = np.empty((batch, n, n))
    for b in range(batch):
        x0, y0 = rng.uniform(-np.pi, np.pi, 2) if b else (np.pi / 2, np.pi / 2)
        dx = (X - x0 + np.pi) % (2 * np.pi) - np.pi
        dy = (Y - y0 + np.pi) % (2 * np.pi) - np.pi
        out[b] = np.exp(-(dx ** 2 + dy ** 2) / (2 * 0.2 ** 2))
    return out


def profiled_traffic(kernel, precision, n, batch):
    """DRAM bytes per launch of `kernel` measured by ncu (dram__bytes_read.sum +
    dram__bytes_write.sum), as recorded in a summary under profiles/ by a line
    ``traffic-per-launch: <kernel> <precision> n=<n> batch=<batch> bytes=<B>``."""
    import re
    pat = re.compile(r"traffic-per-launch:\s+(\S+)\s+(\S+)\s+n=(\d+)\s+batch=(\d+)\s+bytes=(\d+)")
    for f in sorted((ROOT / "profiles").glob("*.md")):
        for line in f.read_text().splitlines():
            m = pat.search(line)
            if m and m.group(1) == kernel and m.group(2) == precision and int(m.group(3)) == n \
                    and int(m.group(4)) == batch:
                return int(m.group(5)), f.name
    return None, None


def profiled_fp64_pipe(kernel, n):
    """FP64-pipe activity (% of peak over the launch, ncu
    sm__pipe_fp64_cycles_active) of an FP64 pass, as recorded in a summary
    under profiles/ by a line ``fp64-pipe-active: <kernel> f64 n=<n> pct=<P>``."""
    import re
    pat = re.compile(r"fp64-pipe-active:\s+(\S+)\s+f64\s+n=(\d+)\s+pct=([0-9.]+)")
    for f in sorted((ROOT / "profiles").glob("*.md")):
        for line in f.read_text().splitlines():
            m = pat.search(line)
            if m and m.group(1) == kernel and int(m.group(2)) == n:
                return float(m.group(3)), f.name
    return None, None


def fft_flops_2d_rhs(nx, ny):
    """FP64 operation count of one 2D right-hand side by the usual FFT
    convention (5 N log2 N flops per complex transform of length N): the
    column pass's 3 transforms per half-spectrum column (forward, two
    inverses) and the row pass's 1.5 per row (two inverses and one forward
    per row pair); the pointwise products (a few percent) are not counted."""
    nkr = nx // 2 + 1
    return 3 * nkr * 5 * ny * math.log2(ny) + 1.5 * ny * 5 * nx * math.log2(nx)


def measure_fma_peak(lib, precision):
    """FMA flops/s of the library's bounded probe kernel on this GPU (None if it fails)."""
    import ctypes as ct
    out = ct.c_double()
    return out.value if lib.ptf_measure_fma_peak(precision, ct.byref(out)) == 0 else None


def load_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms during a region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        lines = Path(self.path).read_text().splitlines()
        os.unlink(self.path)
        return self.summarize(lines)

    @staticmethod
    def summarize(lines):
        """Median SM clock, the maximum clock and every throttle reason seen
        Active, from `FIELDS` rows (csv, noheader, nounits)."""
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in lines:
            r = ln.split(",")
            try:
                sm.append(float(r[1])); smax = float(r[2])
                for nm, val in zip(names, r[5:9]):
                    if val.strip() == "Active":
                        reasons.add(nm)
            except (ValueError, IndexError):
                continue
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def oracle_module():
    import __graft_entry__ as g
    return g._load_module_file("ptf_oracle", ROOT / "oracle" / "ptf_oracle.py")


def oracle_problem(o, n, dt):
    u, v = flow_fns()
    return o.Problem(o.TwoDAdvectingFlow(u=u, v=v), nx=n, Lx=2 * np.pi, kappa=1e-4, eta=1e-4, kappah=1e-12,
                     nkappah=2, dt=dt, stepper="ETDRK4")


def cpu_oracle_rate(args, seconds, max_steps):
    """Time the FP64 oracle (all host cores) on a bounded sample of the workload."""
    o = oracle_module()
    p = oracle_problem(o, args.n, args.dt)
    o.set_c(p, initial_conditions(args.n, 1, 0)[0])
    o.stepforward(p, 1)  # warm-up (plans, caches)
    t0 = time.perf_counter()
    steps = 0
    while steps < max_steps and (time.perf_counter() - t0) < seconds:
        o.stepforward(p, 1)
        steps += 1
    el = time.perf_counter() - t0
    return args.n * args.n * steps / el, steps, el, o.WORKERS


# ---------------------------------------------------------------------------
# GPU comparator: the reference's GPU operation sequence restated with
# torch.fft (cuFFT) and eager elementwise kernels -- what FourierFlows does on
# CUDA.jl for this module: calcN! = two c2r transforms of (i kr s, i l s), the
# product with the flow, one r2c (src/traceradvectiondiffusion.jl:756-769),
# with ETDRK4's stage arithmetic as separate broadcasts.  Not the product;
# reported beside it.
# ---------------------------------------------------------------------------
def etdrk4_tables(torch, Lh, dt, npts=32):
    """Kassam & Trefethen (2005) contour-integral ETDRK4 coefficients (FP64)."""
    r = torch.exp(1j * np.pi * (torch.arange(1, npts + 1, dtype=torch.float64, device=Lh.device) - 0.5) / npts)
    out = {"E": torch.exp(dt * Lh), "E2": torch.exp(dt * Lh / 2)}
    q, f1, f2, f3 = (torch.zeros_like(Lh) for _ in range(4))
    for k in range(npts):
        z = dt * Lh.to(torch.complex128) + r[k]
        ez = torch.exp(z)
        q += ((torch.exp(z / 2) - 1) / z).real
        f1 += ((-4 - z + ez * (4 - 3 * z + z * z)) / z ** 3).real
        f2 += ((2 + z + ez * (z - 2)) / z ** 3).real
        f3 += ((-4 - 3 * z - z * z + ez * (4 - z)) / z ** 3).real
    out.update(Q=dt * q / npts, f1=dt * f1 / npts, f2=dt * f2 / npts, f3=dt * f3 / npts)
    return out


def torch_comparator(torch, n, batch, dt, steps, c0, flush=None, dtype=None):
    dev = "cuda"
    rdt = dtype or torch.float64
    L = 2 * np.pi
    x = torch.tensor(-L / 2 + L / n * np.arange(n), dtype=torch.float64, device=dev)
    Y, X = torch.meshgrid(x, x, indexing="ij")
    u = (4.0 * torch.cos(4 * X) * torch.sin(4 * Y)).to(rdt)
    v = (-4.0 * torch.sin(4 * X) * torch.cos(4 * Y)).to(rdt)
    kr = torch.arange(n // 2 + 1, dtype=torch.float64, device=dev) * (2 * np.pi / L)
    ll = torch.fft.fftfreq(n, d=1.0 / n, dtype=torch.float64, device=dev) * (2 * np.pi / L)
    K2 = kr[None, :] ** 2 + ll[:, None] ** 2
    Lh = -1e-4 * kr[None, :] ** 2 - 1e-4 * ll[:, None] ** 2 - 1e-12 * K2 ** 2
    tb = {k: t.to(rdt) for k, t in etdrk4_tables(torch, Lh, dt).items()}
    ikr = (1j * kr[None, :]).to(torch.complex64 if rdt == torch.float32 else torch.complex128)
    il = (1j * ll[:, None]).to(ikr.dtype)

    def calcN(sh):
        cx = torch.fft.irfft2(ikr * sh, s=(n, n))
        cy = torch.fft.irfft2(il * sh, s=(n, n))
        return torch.fft.rfft2(-(u * cx + v * cy))

    def step(s):
        N1 = calcN(s)
        a = tb["E2"] * s + tb["Q"] * N1
        Na = calcN(a)
        b = tb["E2"] * s + tb["Q"] * Na
        Nb = calcN(b)
        c = tb["E2"] * a + tb["Q"] * (2 * Nb - N1)
        Nc = calcN(c)
        return tb["E"] * s + tb["f1"] * N1 + 2 * tb["f2"] * (Na + Nb) + tb["f3"] * Nc

    s = torch.fft.rfft2(torch.as_tensor(c0, device=dev).reshape(batch, n, n).to(rdt))
    for _ in range(3):
        s = step(s)
    torch.cuda.synchronize()
    ms = 0.0
    for _ in range(steps):
        if flush is not None:
            flush.fill_(1.0)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        s = step(s)
        b.record()
        b.synchronize()
        ms += a.elapsed_time(b)
    return batch * n * n * steps / (ms / 1e3), ms / steps, step, s


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


# Replicas (one process per GPU, no data-path collective): every rank steps
# its own batch of independent solves from its own seed; the only collectives
# are the barrier around the timed region and the max of the ranks' times.
def replica_seed(rank, base=1234):
    return base + rank


# A rank that dies (or never reaches a collective) ends the others' next
# collective with an error after this long, instead of the backend's default.
PG_TIMEOUT_S = 300


def init_ranks(backend, timeout_s=PG_TIMEOUT_S):
    import datetime
    import torch.distributed as dist
    dist.init_process_group(backend, timeout=datetime.timedelta(seconds=timeout_s))


def max_over_ranks(x, world, device):
    """Largest value of x over the ranks (the job's time is its slowest rank's)."""
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(world, units_per_rank, seconds_max):
    """Whole-job throughput: the units all ranks processed over the slowest rank's time."""
    return world * units_per_rank / seconds_max


def run_reference(args):
    world, rank, _ = dist_setup()
    if rank != 0:
        return
    K = max(1, args.steps)
    W = max(0, args.warmup)
    o = oracle_module()
    p = oracle_problem(o, args.n, args.dt)
    o.set_c(p, initial_conditions(args.n, 1, 0)[0])
    o.stepforward(p, W)
    t0 = time.perf_counter()
    o.stepforward(p, K)
    el = time.perf_counter() - t0
    val = args.n * args.n * K / el
    line = {
        "impl": "reference", "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": args.gpus, "steps": K,
        "warmup": W, "ms_per_step": 1e3 * el / K, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": dict(workload(args, 1), precision="FP64 (CPU oracle)"),
        "cpu_baseline": {"value": val, "unit": UNIT, "cores": o.WORKERS, "kind": "port",
                         "sample": f"{K} ETDRK4 steps of one {args.n}x{args.n} solve after {W} warm-up steps "
                                   "(NumPy/pocketfft FP64 restatement; Julia is not available)"},
        "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch
    world, rank, local = dist_setup()
    if world > 1:
        init_ranks("nccl")
    torch.cuda.set_device(local)
    import __graft_entry__ as g
    lib_path = g.PKG_DIR / "libptf.so"
    if not lib_path.exists():
        g.build()
    pkg = g.load_package()
    from ptf_gb300 import _lib as L
    lib = L.load()
    n, B, K, W, dt = args.n, args.batch, args.steps, max(3, args.warmup), args.dt
    u, v = flow_fns()
    kw = dict(nx=n, Lx=2 * np.pi, κ=1e-4, η=1e-4, κh=1e-12, nκh=2, dt=dt, stepper="ETDRK4")

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    def max_ranks(x):
        return max_over_ranks(x, world, "cuda")

    c0 = initial_conditions(n, B, replica_seed(rank))
    # ---------------- FP32 batched ----------------
    p32 = pkg.Problem(pkg.GPU(), pkg.TwoDAdvectingFlow(u=u, v=v), T=np.float32, batch=B, **kw)
    pkg.set_c(p32, c0)
    st32 = torch.cuda.ExternalStream(p32.stream)
    tuning32 = p32.autotune(trial_steps=4) if not args.no_tune else p32.tuning
    pkg.stepforward(p32, W)
    sampler = ClockSampler(torch.cuda.current_device())
    sampler.start()
    time.sleep(0.3)
    barrier()
    launches0 = p32.kernel_launches
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st32)
    pkg.stepforward(p32, K)
    e1.record(st32)
    e1.synchronize()
    barrier()
    ms32 = max_ranks(e0.elapsed_time(e1))
    launches = p32.kernel_launches - launches0
    value = job_rate(world, B * n * n * K, ms32 / 1e3)
    # per-pass roofline (CUDA events around each pass; one branch, so that
    # the events of concurrent passes do not overlap)
    p32.tuning = dict(branches=1, solves_per_group=0)
    lib.ptf_profile(p32._h, 1)
    pkg.stepforward(p32, K)
    prof = {}
    for kind, name in ((0, "column_pass"), (1, "row_pass")):
        ms, cnt, by = ct_read(lib, p32._h, kind)
        prof[name] = {"ms": ms, "launches": cnt, "bytes": by}
    lib.ptf_profile(p32._h, 0)
    p32.tuning = {k: v for k, v in tuning32.items() if k != "ms_per_step"}
    # ---------------- FP64 plain ----------------
    p64 = pkg.Problem(pkg.GPU(), pkg.TwoDAdvectingFlow(u=u, v=v), T=np.float64, batch=1, **kw)
    pkg.set_c(p64, c0[0])
    st64 = torch.cuda.ExternalStream(p64.stream)
    tuning64 = p64.autotune(trial_steps=4) if not args.no_tune else p64.tuning
    pkg.stepforward(p64, W)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MB > L2
    K64 = K
    barrier()
    evs = []
    with torch.cuda.stream(st64):
        for _ in range(K64):
            flush.fill_(1.0)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(st64)
            pkg.stepforward(p64, 1)
            b.record(st64)
            evs.append((a, b))
    torch.cuda.synchronize()
    ms64 = max_ranks(sum(a.elapsed_time(b) for a, b in evs))
    value64 = world * n * n * K64 / (ms64 / 1e3)
    lib.ptf_profile(p64._h, 1)
    pkg.stepforward(p64, 8)
    prof64 = {}
    for kind, name in ((0, "column_pass"), (1, "row_pass")):
        ms, cnt, by = ct_read(lib, p64._h, kind)
        prof64[name] = {"ms": ms, "launches": cnt, "bytes": by}
    lib.ptf_profile(p64._h, 0)
    clocks = sampler.stop()
    # FP64 roof: the FP64 FMA rate of this GPU, measured by the library's probe
    fp64_peak = measure_fma_peak(lib, 0)
    fp64_flops_step = 4 * fft_flops_2d_rhs(n, n)
    fp64_achieved = fp64_flops_step / (ms64 / K64 / 1e3)
    bytes64_step = sum(x["bytes"] for x in prof64.values()) / 8  # 8 profiled steps
    roof64 = {"bound": "fp64", "achieved": fp64_achieved / 1e12, "unit": "TFLOP/s",
              "peak": fp64_peak / 1e12 if fp64_peak else None,
              "peak_kind": "measured (ptf_measure_fma_peak, 2 flops per DFMA)",
              "frac": (fp64_achieved / fp64_peak) if fp64_peak else None,
              "flops_per_step": fp64_flops_step,
              "flop_model": "5 N log2 N per complex FFT; 3 column + 1.5 row transforms per line per RHS; 4 RHS/step",
              "hbm_GBps_algorithmic": bytes64_step / (ms64 / K64 / 1e3) / 1e9}
    # the FP64 pipe's measured activity in the same passes (the flop model
    # above counts a radix-2 FFT's operations; the radix-16 transforms issue
    # fewer, so the pipe is busier than `frac` suggests)
    pipe = {k: profiled_fp64_pipe(k, n) for k in ("column_pass", "row_pass")}
    if all(v[0] is not None for v in pipe.values()):
        roof64["fp64_pipe_active_pct_ncu"] = {k: v[0] for k, v in pipe.items()}
        roof64["fp64_pipe_source"] = pipe["column_pass"][1]
    # ---------------- accuracy vs the FP64 oracle ----------------
    # The bench's own problems, restarted from the initial condition and
    # stepped over the configured 1000 steps (t = 0.5 at dt = 5e-4); solve 0
    # (the Gaussian at (pi/2, pi/2), a cell centre of the flow) is compared
    # with the FP64 oracle.
    acc = {}
    if rank == 0 and not args.no_oracle_check:
        o = oracle_module()
        nacc = int(round(args.acc_time / dt))
        pkg.set_c(p32, c0)
        pkg.stepforward(p32, nacc)
        pkg.updatevars(p32)
        pkg.set_c(p64, c0[0])
        pkg.stepforward(p64, nacc)
        pkg.updatevars(p64)
        c32 = p32.vars.c[0].copy()
        c64 = p64.vars.c.copy()
        po = oracle_problem(o, n, dt)
        o.set_c(po, c0[0])
        t0 = time.perf_counter()
        o.stepforward(po, nacc)
        o.updatevars(po)
        m0 = float(c0[0].sum())
        acc = {
            "steps": nacc, "t": nacc * dt,
            "rel_l2_fp32_vs_oracle": o.rel_l2(c32, po.vars.c),
            "rel_l2_fp64_vs_oracle": o.rel_l2(c64, po.vars.c),
            "mass_drift_fp32": float(c32.sum()) / m0 - 1,
            "mass_drift_fp64": float(c64.sum()) / m0 - 1,
            "mass_drift_oracle": float(po.vars.c.sum()) / m0 - 1,
            "oracle_seconds": time.perf_counter() - t0,
        }
    # ---------------- torch/cuFFT restatement of the reference's GPU sequence ----------------
    comparator = None
    if rank == 0 and not args.no_comparator:
        try:
            KC = max(3, min(K, 20))
            v32, ms32c, _, _ = torch_comparator(torch, n, B, dt, KC, c0, dtype=torch.float32)
            v64c, ms64c, step64, _ = torch_comparator(torch, n, 1, dt, KC, c0[0], flush=flush)
            # same algorithm: a fresh FP64 comparator solve against a fresh FP64 solve of ours, 3 steps
            s = torch.fft.rfft2(torch.as_tensor(c0[0], device="cuda").reshape(1, n, n))
            for _ in range(3):
                s = step64(s)
            cref = torch.fft.irfft2(s, s=(n, n))[0].cpu().numpy()
            q = pkg.Problem(pkg.GPU(), pkg.TwoDAdvectingFlow(u=u, v=v), T=np.float64, batch=1, **kw)
            pkg.set_c(q, c0[0])
            pkg.stepforward(q, 3)
            pkg.updatevars(q)
            agree = float(np.linalg.norm(q.vars.c - cref) / np.linalg.norm(cref))
            del q
            comparator = {
                "what": "reference GPU op sequence restated in torch.fft (cuFFT) + eager elementwise kernels",
                "fp32_batched": {"value": v32, "unit": UNIT, "ms_per_step": ms32c, "batch": B},
                "fp64_plain": {"value": v64c, "unit": UNIT, "ms_per_step": ms64c, "batch": 1},
                "steps": KC, "rel_l2_fp64_vs_ours_3_steps": agree,
                "ours_over_comparator_fp32": value / v32, "ours_over_comparator_fp64": value64 / v64c,
            }
        except Exception as e:
            comparator = {"error": f"{type(e).__name__}: {e}"}
        torch.cuda.empty_cache()
    # ---------------- end to end through the public API ----------------
    S = min(25, K)
    frames = max(1, K // S)
    pin_in = torch.empty((B, n, n), dtype=torch.float64, pin_memory=True)
    pin_in.numpy()[...] = c0
    pin_out = torch.empty((B, n, n), dtype=torch.float64, pin_memory=True)
    p32.vars.c = pin_out.numpy()
    barrier()
    t0 = time.perf_counter()
    pkg.set_c(p32, pin_in.numpy())
    for _ in range(frames):
        pkg.stepforward(p32, S)
        pkg.updatevars(p32)
    t1 = time.perf_counter()
    e2e_s = max_ranks(t1 - t0)
    e2e_val = job_rate(world, B * n * n * frames * S, e2e_s)
    bytes_field = B * n * n * 8
    # ---------------- other configurations (rank 0, bounded) ----------------
    workloads = run_workloads(args, pkg, torch) if rank == 0 and not args.only_main else {}
    # ---------------- CPU baseline (rank 0) ----------------
    return _finish_ours(args, world, rank, value, ms32, K, W, B, n, dt, launches, prof, prof64, tuning32, tuning64,
                        value64, ms64, K64, roof64, acc, comparator, e2e_val, frames, S, bytes_field, clocks, workloads)


def run_workloads(args, pkg, torch):
    """The secondary configurations (rank 0): each entry carries its own
    timing, accuracy and the seconds it took; a failure is reported in place."""
    workloads = {}
    for key, fn in (("2d_cellular_4096", lambda: run_config2_4096(pkg, torch, args.config_steps_2d)),
                    ("3d_abc_256", lambda: run_abc3d_256(pkg, torch, args.config_steps_3d)),
                    ("ensemble_256_solves", lambda: run_ensemble_256(pkg, torch, args.ensemble_steps)),
                    ("ensemble_256_solves_clock_t",
                     lambda: run_ensemble_256(pkg, torch, args.ensemble_steps, time_mode="clock",
                                              fp64_check=False)),
                    ("served_fp32", lambda: run_served_stream(pkg, np.float32, args.serve_requests, args.serve_rate)),
                    ("served_fp64", lambda: run_served_stream(pkg, np.float64, args.serve_requests_fp64,
                                                        args.serve_rate / 8, check=0))):
        if args.only and key not in args.only.split(","):
            continue
        try:
            t_w = time.perf_counter()
            workloads[key] = fn()
            workloads[key]["bench_seconds"] = time.perf_counter() - t_w
        except Exception as e:  # report the failure in the line rather than losing the main result
            workloads[key] = {"error": f"{type(e).__name__}: {e}"}
    return workloads


def _finish_ours(args, world, rank, value, ms32, K, W, B, n, dt, launches, prof, prof64, tuning32, tuning64,
                 value64, ms64, K64, roof64, acc, comparator, e2e_val, frames, S, bytes_field, clocks, workloads):
    import torch
    cpu = None
    if rank == 0 and not args.no_cpu:
        rate, steps, el, cores = cpu_oracle_rate(args, args.cpu_seconds, 200)
        cpu = {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"{steps} ETDRK4 steps of one {n}x{n} FP64 solve ({el:.1f} s, NumPy/pocketfft restatement)"}
    if rank != 0:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return
    hbm_peak, peak_kind = load_peaks()
    dom = max(prof, key=lambda k: prof[k]["ms"])
    d = prof[dom]
    achieved = d["bytes"] / (d["ms"] / 1e3) / 1e9
    traffic, traffic_src = profiled_traffic(dom, "f32", n, B)
    roof = {"bound": "hbm", "kernel": f"{dom} (FP32, {n}x{n}, batch {B})", "achieved": achieved, "peak": hbm_peak,
            "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / hbm_peak,
            "traffic": traffic, "traffic_source": traffic_src,
            "traffic_over_algorithmic": (traffic / (d["bytes"] / max(1, d["launches"]))) if traffic else None,
            "avg_launch_us": 1e3 * d["ms"] / max(1, d["launches"]),
            "algorithmic_bytes_per_launch": d["bytes"] / max(1, d["launches"]),
            "share_of_step": d["ms"] / sum(x["ms"] for x in prof.values())}
    passes = {k: {"ms_per_launch": x["ms"] / max(1, x["launches"]), "GBps": x["bytes"] / (x["ms"] / 1e3) / 1e9,
                  "launches": x["launches"]} for k, x in prof.items()}
    passes64 = {k: {"ms_per_launch": x["ms"] / max(1, x["launches"]), "GBps": x["bytes"] / (x["ms"] / 1e3) / 1e9,
                    "launches": x["launches"]} for k, x in prof64.items()}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
        "ms_per_step": ms32 / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded Gaussian ensemble on the cellular flow)",
        "config": dict(workload(args, B), parallelism="replicas" if world > 1 else "single GPU"),
        "tuning": {"fp32_batched": tuning32, "fp64_plain": tuning64},
        "fp64_plain": {"value": value64, "unit": UNIT, "ms_per_step": ms64 / K64, "steps": K64, "dtype": "f64",
                       "passes": passes64, "ratio_fp32_batched_over_fp64": value / value64, "roofline": roof64,
                       "hbm_frac": roof64["hbm_GBps_algorithmic"] / hbm_peak},
        "accuracy": acc,
        "gpu_comparator": comparator,
        "passes": passes,
        "roofline": roof,
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": bytes_field / (frames * S),
                "d2h_bytes_per_step": bytes_field / S,
                "api": f"set_c(pinned host) + {frames} x (stepforward({S}) + updatevars(pinned host))"},
        "gpu_launches": launches,
        "clocks": clocks,
        "serving": ({k: workloads["served_fp32"].get(k) for k in ("p50_latency_s", "p99_latency_s", "grid_pt_steps_per_s",
                                                               "requests", "completed")}
                    if "served_fp32" in workloads else None),
        "workloads": workloads,
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


# ---------------------------------------------------------------------------
# Secondary configurations (bounded samples; reported inside the one JSON line)
# ---------------------------------------------------------------------------
def _timed_run(pkg, torch, p, c0, steps, warm=3):
    """set_c, `warm` untimed steps (graph capture), set_c again, then exactly
    `steps` steps timed with CUDA events on the problem's stream; returns
    (ms per step, vars.c after the `steps` steps)."""
    st = torch.cuda.ExternalStream(p.stream)
    pkg.set_c(p, c0)
    pkg.stepforward(p, warm)
    pkg.set_c(p, c0)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    pkg.stepforward(p, steps)
    e1.record(st)
    e1.synchronize()
    pkg.updatevars(p)
    return e0.elapsed_time(e1) / steps, p.vars.c.copy()


def _window(pkg, p, c0, steps):
    pkg.set_c(p, c0)
    pkg.stepforward(p, steps)
    pkg.updatevars(p)
    return p.vars.c.copy()


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _drift(c, m0):
    return float(np.sum(c)) / m0 - 1.0


def _bounded(c, c0):
    """A result that stayed a tracer field: finite, and no larger than twice
    the initial maximum (advection-diffusion keeps max|c| <= max|c0|; small
    spectral over- and undershoots aside)."""
    return bool(np.all(np.isfinite(c))) and float(np.abs(c).max()) <= 2.0 * float(np.abs(c0).max())


RK4_REAL_AXIS_LIMIT = 2.785  # RK4's stability interval on the negative real axis: dt*|L| <= 2.785


def run_config2_4096(pkg, torch, steps=1000, oracle_steps=20, dt=1e-4):
    """2D cellular flow at 4096², ETDRK4, κ=η=1e-4, κh=1e-12 (nκh=2), Gaussian
    σ=0.2 at (π/2, π/2): one FP32 and one FP64 solve of the configured 1000
    steps (dt = 1e-4 for an advective CFL number of 0.82; the configured 2e-3
    gives 16 and every solution diverges), FP32 against the FP64 GPU path at
    full length, and both against the FP64 oracle over the first
    `oracle_steps` steps at full size."""
    n = 4096
    u, v = flow_fns()
    kw = dict(nx=n, Lx=2 * np.pi, κ=1e-4, η=1e-4, κh=1e-12, nκh=2, dt=dt, stepper="ETDRK4")
    x = -np.pi + 2 * np.pi / n * np.arange(n)
    X, Y = np.meshgrid(x, x)
    c0 = np.exp(-((X - np.pi / 2) ** 2 + (Y - np.pi / 2) ** 2) / (2 * 0.2 ** 2))
    m0 = float(c0.sum())
    out, full, win = {}, {}, {}
    for T, name in ((np.float32, "fp32"), (np.float64, "fp64")):
        p = pkg.Problem(pkg.GPU(), pkg.TwoDAdvectingFlow(u=u, v=v), T=T, **kw)
        ms, full[name] = _timed_run(pkg, torch, p, c0, steps)
        win[name] = _window(pkg, p, c0, oracle_steps)
        out[name] = {"ms_per_step": ms, "grid_pt_steps_per_s": n * n / (ms / 1e3),
                     "mass_drift": _drift(full[name], m0), "device_bytes": p.device_bytes}
        del p
        torch.cuda.empty_cache()
    o = oracle_module()
    r = o.Problem(o.TwoDAdvectingFlow(u=u, v=v), nx=n, Lx=2 * np.pi, kappa=1e-4, eta=1e-4, kappah=1e-12,
                  nkappah=2, dt=dt, stepper="ETDRK4")
    t0 = time.perf_counter()
    o.set_c(r, c0)
    o.stepforward(r, oracle_steps)
    o.updatevars(r)
    out.update({
        "steps": steps, "dt": dt, "nominal_dt": 0.002,
        "rel_l2_fp32_vs_fp64_gpu": _rel(full["fp32"], full["fp64"]),
        "oracle_window": {"steps": oracle_steps, "rel_l2_fp64_vs_oracle": _rel(win["fp64"], r.vars.c),
                          "rel_l2_fp32_vs_oracle": _rel(win["fp32"], r.vars.c),
                          "mass_drift_fp64": _drift(win["fp64"], m0), "mass_drift_fp32": _drift(win["fp32"], m0),
                          "mass_drift_oracle": _drift(r.vars.c, m0), "oracle_seconds": time.perf_counter() - t0},
        "ratio_fp32_over_fp64": out["fp32"]["grid_pt_steps_per_s"] / out["fp64"]["grid_pt_steps_per_s"],
        "workload": "2D cellular psi=cos(4x)cos(4y) 4096^2, ETDRK4, kappa=eta=1e-4, kappah=1e-12 nkappah=2, "
                    f"dt={dt:g} (CFL 0.82)",
    })
    return out


def run_abc3d_256(pkg, torch, steps=500, oracle_steps=20):
    """3D ABC flow, 256³, ETDRK4, κ=η=ι=5e-4, dt=0.005, Gaussian σ=0.3 at the
    centre: FP32 and FP64 single solves of the configured 500 steps, FP32
    against the FP64 GPU path at full length, and both against the FP64
    oracle over the first `oracle_steps` steps at full size."""
    n, dt = 256, 0.005
    A, B, C = 1.0, np.sqrt(2 / 3), np.sqrt(1 / 3)
    u = lambda x, y, z: A * np.sin(z) + C * np.cos(y)
    v = lambda x, y, z: B * np.sin(x) + A * np.cos(z)
    w = lambda x, y, z: C * np.sin(y) + B * np.cos(x)
    x = -np.pi + 2 * np.pi / n * np.arange(n)
    Z, Y, X = np.meshgrid(x, x, x, indexing="ij")
    c0 = np.exp(-(X ** 2 + Y ** 2 + Z ** 2) / (2 * 0.3 ** 2))
    del X, Y, Z
    m0 = float(c0.sum())
    out, full, win = {}, {}, {}
    for T, name in ((np.float32, "fp32"), (np.float64, "fp64")):
        t0 = time.perf_counter()
        p = pkg.Problem(pkg.GPU(), pkg.ThreeDAdvectingFlow(u=u, v=v, w=w), nx=n, κ=5e-4, dt=dt,
                        stepper="ETDRK4", T=T)
        setup = time.perf_counter() - t0
        ms, full[name] = _timed_run(pkg, torch, p, c0, steps)
        win[name] = _window(pkg, p, c0, oracle_steps)
        out[name] = {"ms_per_step": ms, "grid_pt_steps_per_s": n ** 3 / (ms / 1e3), "setup_s": setup,
                     "mass_drift": _drift(full[name], m0), "device_bytes": p.device_bytes}
        del p
        torch.cuda.empty_cache()
    o = oracle_module()
    r = o.Problem(o.ThreeDAdvectingFlow(u=u, v=v, w=w), nx=n, kappa=5e-4, dt=dt, stepper="ETDRK4")
    t0 = time.perf_counter()
    o.set_c(r, c0)
    o.stepforward(r, oracle_steps)
    o.updatevars(r)
    out.update({
        "steps": steps, "rel_l2_fp32_vs_fp64_gpu": _rel(full["fp32"], full["fp64"]),
        "oracle_window": {"steps": oracle_steps, "rel_l2_fp64_vs_oracle": _rel(win["fp64"], r.vars.c),
                          "rel_l2_fp32_vs_oracle": _rel(win["fp32"], r.vars.c),
                          "mass_drift_fp64": _drift(win["fp64"], m0), "mass_drift_fp32": _drift(win["fp32"], m0),
                          "mass_drift_oracle": _drift(r.vars.c, m0), "oracle_seconds": time.perf_counter() - t0},
        "workload": "3D ABC flow 256^3, ETDRK4, kappa=eta=iota=5e-4, dt=0.005, Gaussian sigma=0.3 at the centre",
    })
    return out


def run_ensemble_256(pkg, torch, steps, seed=2024, time_mode="stage", fp64_check=True, oracle_solves=4):
    """Batched ensemble: 256 2D solves, n uniform in {64,128,256,512}, κ
    log-uniform in [1e-4,1e-2], ψ = cos(x + 0.3 sin t) cos y re-evaluated at
    every RK4 stage (time_mode "stage") or frozen at clock.t for the step as
    the reference does ("clock"), Gaussian blobs (random centres, σ ∈
    [0.1,0.5]), RK4, dt=0.005, FP32 with each solve's (0,0) mode in FP64; a
    row and a column launch per stage, steps from a CUDA graph.  Every
    solve's result is compared with the same ensemble run by the FP64
    batched engine (the oracle for all 256 solves of 1000 steps would take
    hours of CPU), and the `oracle_solves` smallest-κ 64² solves with the
    FP64 oracle; mass drift of every solve against its FP64 twin."""
    rng = np.random.default_rng(seed)
    sizes = rng.choice([64, 128, 256, 512], size=256)
    cases = []
    for n in sizes:
        n = int(n)
        κ = float(10 ** rng.uniform(-4, -2))
        x0, y0 = rng.uniform(-np.pi, np.pi, 2)
        sig = float(rng.uniform(0.1, 0.5))
        cases.append((n, κ, initial_gaussian(n, x0, y0, sig)))

    def spec(n, κ):
        return pkg.SolveSpec(n=n, nsteps=steps, dt=0.005, kappa=κ, flow="cellular", time_mode=time_mode,
                             U=1.0, eps=0.3, omega=1.0, Kx=1, Ky=1)

    def run(T):
        b = pkg.BatchedProblem(T=T, slots_per_bucket=96)
        t0 = time.perf_counter()
        ids = [b.add(spec(n, κ), c0) for n, κ, c0 in cases]
        setup = time.perf_counter() - t0
        st = torch.cuda.ExternalStream(b.stream)
        b.synchronize()
        l0 = b.info()["kernel_launches"]
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        b.step(steps)  # the first step captures the graph: inside the timed region
        e1.record(st)
        e1.synchronize()
        b.synchronize()
        ms = e0.elapsed_time(e1)
        info = b.info()
        fields = [b.get_c(i) for i in ids]
        b.close()
        torch.cuda.empty_cache()
        return ms, setup, (info["kernel_launches"] - l0) / steps, info["device_bytes"], fields

    ms, setup, lps, dev_bytes, f32 = run(np.float32)
    pts = float(sum(n * n for n, _, _ in cases))
    m0 = [float(c0.sum()) for _, _, c0 in cases]
    # solves whose diffusive eigenvalue dt*kappa*|k|^2_max lies beyond RK4's
    # real-axis stability limit: they diverge in any precision (the FP64
    # oracle included) and are left out of the accuracy statistics
    unstable = [i for i, (n, κ, _) in enumerate(cases) if 0.005 * κ * 2 * (n / 2) ** 2 > RK4_REAL_AXIS_LIMIT]
    ok = [i for i in range(len(cases)) if i not in unstable]
    res = {"solves": len(cases), "sizes": {str(k): int((sizes == k).sum()) for k in (64, 128, 256, 512)},
           "steps": steps, "ms_per_step": ms / steps, "grid_pt_steps_per_s": pts * steps / (ms / 1e3),
           "setup_s": setup, "launches_per_step": lps, "device_bytes": dev_bytes,
           "rk4_unstable_solves": {"count": len(unstable), "criterion": "dt*kappa*|k|^2_max > 2.785 (RK4 real-axis "
                                   "limit) at dt=0.005: 512^2 solves with kappa > 4.2e-3; they diverge in every "
                                   "precision and are excluded from the accuracy figures",
                                   "diverged_fp32": int(sum(not _bounded(f32[i], cases[i][2]) for i in unstable))},
           "stable_solves_bounded_fp32": int(sum(_bounded(f32[i], cases[i][2]) for i in ok)),
           "mass_drift_fp32_max_abs": max(abs(_drift(f32[i], m0[i])) for i in ok),
           "workload": f"256 solves n in {{64..512}}, RK4 dt=0.005, {steps} steps, cellular psi=cos(x+0.3 sin t)cos y at "
                       f"{'stage times' if time_mode == 'stage' else 'clock.t (frozen per step)'}, FP32 with FP64 k=0 mode"}
    if fp64_check:
        ms64, _, _, _, f64 = run(np.float64)
        rel = [_rel(f32[i], f64[i]) for i in ok]
        dd = [abs(_drift(f32[i], m0[i]) - _drift(f64[i], m0[i])) for i in ok]
        res["fp64_batched"] = {"ms_per_step": ms64 / steps, "grid_pt_steps_per_s": pts * steps / (ms64 / 1e3),
                               "stable_solves_bounded": int(sum(_bounded(f64[i], cases[i][2]) for i in ok)),
                               "unstable_solves_diverged": int(sum(not _bounded(f64[i], cases[i][2])
                                                                   for i in unstable))}
        res["rel_l2_fp32_vs_fp64_gpu"] = {"solves": len(rel), "max": max(rel), "median": float(np.median(rel)),
                                          "solves_over_1e-5": int(sum(r > 1e-5 for r in rel))}
        res["mass_drift_fp32_minus_fp64_max_abs"] = max(dd)
        res["mass_drift_fp64_max_abs"] = max(abs(_drift(f64[i], m0[i])) for i in ok)
    if oracle_solves:
        o = oracle_module()
        picks = sorted([i for i, (n, _, _) in enumerate(cases) if n == 64], key=lambda i: cases[i][1])[:oracle_solves]
        uu = lambda x, y, t: np.cos(x + 0.3 * np.sin(t)) * np.sin(y)
        vv = lambda x, y, t: -np.sin(x + 0.3 * np.sin(t)) * np.cos(y)
        errs, drifts = [], []
        t0 = time.perf_counter()
        for i in picks:
            n, κ, c0 = cases[i]
            r = o.Problem(o.TwoDAdvectingFlow(u=uu, v=vv, steadyflow=False), nx=n, kappa=κ, dt=0.005,
                          stage_time=(time_mode == "stage"))
            o.set_c(r, c0)
            o.stepforward(r, steps)
            o.updatevars(r)
            errs.append(_rel(f32[i], r.vars.c))
            drifts.append(abs(_drift(f32[i], m0[i]) - _drift(r.vars.c, m0[i])))
        res["oracle_check"] = {"solves": [f"64^2 kappa={cases[i][1]:.2e}" for i in picks], "steps": steps,
                               "rel_l2_fp32_vs_oracle": errs, "mass_drift_vs_oracle_max_abs": max(drifts),
                               "oracle_seconds": time.perf_counter() - t0}
    return res


def initial_gaussian(n, x0, y0, sig, L=2 * np.pi):
    x = -L / 2 + L / n * np.arange(n)
    Y, X = np.meshgrid(x, x, indexing="ij")
    dx = (X - x0 + L / 2) % L - L / 2
    dy = (Y - y0 + L / 2) % L - L / 2
    return np.exp(-(dx ** 2 + dy ** 2) / (2 * sig ** 2))


def random_phase_flow(n, rng, dim=2, kmin=4, kmax=16, L=2 * np.pi):
    """Incompressible random flow: 2D from a streamfunction with random-phase
    modes 4 ≤ |k| ≤ 16, |û| ∝ |k|^-3 (|ψ̂| ∝ |k|^-4); 3D as the curl of a random
    vector potential with the same spectrum; rms speed normalised to 1."""
    k1 = np.fft.fftfreq(n, 1.0 / n)
    kr = np.arange(n // 2 + 1)
    if dim == 2:
        l, k = np.meshgrid(k1, kr, indexing="ij")
        K = np.sqrt(k ** 2 + l ** 2)
        mask = (K >= kmin) & (K <= kmax)
        amp = np.where(mask, np.maximum(K, 1) ** -4.0, 0.0)
        psih = amp * np.exp(2j * np.pi * rng.random(K.shape))
        u = np.fft.irfft2(-1j * l * psih, s=(n, n))
        v = np.fft.irfft2(1j * k * psih, s=(n, n))
        rms = np.sqrt(np.mean(u ** 2 + v ** 2))
        return u / rms, v / rms
    m, l, k = np.meshgrid(k1, k1, kr, indexing="ij")
    K = np.sqrt(k ** 2 + l ** 2 + m ** 2)
    mask = (K >= kmin) & (K <= kmax)
    amp = np.where(mask, np.maximum(K, 1) ** -4.0, 0.0)
    Ah = [amp * np.exp(2j * np.pi * rng.random(K.shape)) for _ in range(3)]
    s = (n, n, n)
    u = np.fft.irfftn(1j * (l * Ah[2] - m * Ah[1]), s=s, axes=(0, 1, 2))
    v = np.fft.irfftn(1j * (m * Ah[0] - k * Ah[2]), s=s, axes=(0, 1, 2))
    w = np.fft.irfftn(1j * (k * Ah[1] - l * Ah[0]), s=s, axes=(0, 1, 2))
    rms = np.sqrt(np.mean(u ** 2 + v ** 2 + w ** 2))
    return u / rms, v / rms, w / rms


def run_served_stream(pkg, T, nreq, rate, seed=5150, pool=8, check=8, max_queued=256):
    """Served stream: requests with Poisson arrivals at `rate` per second; each
    a 2D grid from {64²..1024²} or 3D 128³ (one in ten), steps log-uniform in
    [100,5000], κ log-uniform in [1e-4,1e-2], random-phase incompressible
    flow (|k| in [4,16], |û| ∝ |k|^-3, rms 1); dt per request for an advective
    CFL of 0.5 and a diffusive number of 1 (RK4).  Flows come from a seeded
    pool of `pool` per grid size (input generation is not what is measured).
    The feeder holds back while `max_queued` requests wait (bounded host
    memory; counted in `feeder_holds`).  Every result's mass drift comes from
    the server's per-request record; `check` seeded requests (n <= 256) are
    re-run alone through an FP64 single-solve handle and compared."""
    import threading
    rng = np.random.default_rng(seed)
    t_prep = time.perf_counter()
    flows = {}
    for n in (64, 128, 256, 512, 1024):
        flows[(2, n)] = [random_phase_flow(n, rng, dim=2) for _ in range(pool)]
    flows[(3, 128)] = [random_phase_flow(128, rng, dim=3) for _ in range(max(2, pool // 2))]
    reqs = []
    for i in range(nreq):
        three = rng.random() < 0.1
        n = 128 if three else int(rng.choice([64, 128, 256, 512, 1024]))
        nsteps = int(10 ** rng.uniform(2, np.log10(5000)))
        κ = float(10 ** rng.uniform(-4, -2))
        fl = flows[(3 if three else 2, n)]
        k = int(rng.integers(len(fl)))
        umax = max(float(np.abs(f).max()) for f in fl[k])
        kmax = n / 2
        dt = min(0.5 / (umax * kmax), 1.0 / (κ * (3 if three else 2) * kmax ** 2))
        x0 = rng.uniform(-np.pi, np.pi, 3)
        sig = float(rng.uniform(0.1, 0.5))
        reqs.append((three, n, nsteps, κ, dt, k, x0, sig))
    prep = time.perf_counter() - t_prep
    x128 = -np.pi + 2 * np.pi / 128 * np.arange(128)
    Z, Y, X = np.meshgrid(x128, x128, x128, indexing="ij")
    r3 = X ** 2 + Y ** 2 + Z ** 2
    del X, Y, Z

    def inputs(req):
        three, n, nsteps, κ, dt, k, x0, sig = req
        spec = pkg.SolveSpec(n=n, dim=3 if three else 2, nsteps=nsteps, dt=dt, kappa=κ)
        c0 = np.exp(-r3 / (2 * sig ** 2)) if three else initial_gaussian(n, x0[0], x0[1], sig)
        return spec, c0, flows[(3 if three else 2, n)][k]

    srv = pkg.Server(T=T, chunk_steps=50, slots_per_bucket=32)
    gaps = rng.exponential(1.0 / rate, size=nreq)
    ids = [None] * nreq
    holds = [0]

    def feeder():
        t_next = time.perf_counter()
        for i, (req, g) in enumerate(zip(reqs, gaps)):
            t_next += g
            dt_wait = t_next - time.perf_counter()
            if dt_wait > 0:
                time.sleep(dt_wait)
            while srv.stats()["queued"] >= max_queued:
                holds[0] += 1
                time.sleep(0.01)
            spec, c0, flow = inputs(req)
            ids[i] = srv.submit(spec, c0, *flow)

    t0 = time.perf_counter()
    th = threading.Thread(target=feeder)
    th.start()
    th.join()
    srv.wait_all(7200)
    wall = time.perf_counter() - t0
    st = srv.stats()
    drifts, diverged = [], []
    for i, rid in enumerate(ids):
        _, c = srv.poll(rid)
        if _bounded(c, inputs(reqs[i])[1]):
            drifts.append(srv.result_info(rid)["mass_drift"])
        else:
            three, n, nsteps, κ, dt, _, _, _ = reqs[i]
            diverged.append({"dim": 3 if three else 2, "n": n, "steps": nsteps, "kappa": κ, "dt": dt})
    chk = {}
    diverged_keys = {(d["n"], d["steps"], d["kappa"]) for d in diverged}
    if check:
        picks = [i for i in range(nreq) if reqs[i][1] <= 256 and not reqs[i][0]
                 and (reqs[i][1], reqs[i][2], reqs[i][3]) not in diverged_keys][:check]  # bounded requests only
        errs, dd = [], []
        for i in picks:
            spec, c0, (u, v) = inputs(reqs[i])
            _, c = srv.poll(ids[i])
            p = pkg.Problem(pkg.GPU(), pkg.TwoDAdvectingFlow(), nx=spec.n, κ=spec.kappa, η=spec.kappa, dt=spec.dt,
                            T=np.float64)
            p.set_flow_arrays(u, v)
            pkg.set_c(p, c0)
            pkg.stepforward(p, spec.nsteps)
            pkg.updatevars(p)
            errs.append(_rel(c, p.vars.c))
            m0 = float(c0.sum())
            dd.append(abs(_drift(c, m0) - _drift(p.vars.c, m0)))
            del p
        # the smallest diverged 2D request, run by the FP64 CPU oracle: it diverges there too
        small = sorted([i for i in range(nreq) if not reqs[i][0] and reqs[i][1] <= 128
                        and (reqs[i][1], reqs[i][2], reqs[i][3]) in diverged_keys],
                       key=lambda i: reqs[i][1] * reqs[i][2])
        if small:
            i = small[0]
            spec, c0, (u, v) = inputs(reqs[i])
            o = oracle_module()
            r = o.Problem(o.TwoDAdvectingFlow(u=lambda *a: u, v=lambda *a: v), nx=spec.n, kappa=spec.kappa,
                          dt=spec.dt)
            o.set_c(r, c0)
            o.stepforward(r, spec.nsteps)
            o.updatevars(r)
            chk["oracle_on_a_diverged_request"] = {"n": spec.n, "steps": spec.nsteps, "kappa": spec.kappa,
                                                   "oracle_bounded": _bounded(r.vars.c, c0)}
        chk.update({"requests": len(picks), "what": "result vs the same request run alone by an FP64 single-solve handle",
               "rel_l2_max": max(errs) if errs else None, "rel_l2_median": float(np.median(errs)) if errs else None,
               "mass_drift_diff_max_abs": max(dd) if dd else None})
    srv.close()
    work = sum(r[1] ** (3 if r[0] else 2) * r[2] for r in reqs)
    return {"requests": nreq, "arrival_rate_per_s": rate, "completed": st["completed"], "failed": st["failed"],
            "p50_latency_s": st["p50_s"], "p99_latency_s": st["p99_s"], "mean_latency_s": st["mean_s"],
            "grid_pt_steps_per_s": st["grid_point_steps"] / wall, "wall_s": wall, "total_grid_pt_steps": work,
            "peak_device_bytes": st["device_bytes"], "input_prep_s": prep, "feeder_holds": holds[0],
            "server_time": {"admission_s": st["admit_s"], "stepping_s": st["chunk_s"], "chunks": st["chunks"],
                            "what": "worker wall time admitting requests and stepping chunks (launch to completion)"},
            "mass_drift_max_abs": max(abs(d) for d in drifts), "mass_drift_median_abs": float(np.median(np.abs(drifts))),
            "diverged": {"count": len(diverged), "examples": diverged[:6],
                         "why": "under-resolved: the advective form, like the reference's, is not dealiased; "
                                "at kappa near 1e-4 on small grids the tracer is thinned below the grid scale "
                                "and the aliasing instability grows in every precision (mass drift and the "
                                "FP64 check are over the bounded results)"},
            "fp64_check": chk,
            "mix": "2D n in {64..1024} (90%), 3D 128^3 (10%); steps log-uniform [100,5000]; kappa log-uniform "
                   f"[1e-4,1e-2]; RK4; flows from a seeded pool of {pool} per size"}


def ct_read(lib, h, kind):
    import ctypes as ct
    ms, cnt, by = ct.c_double(), ct.c_int64(), ct.c_double()
    rc = lib.ptf_profile_read(h, kind, ct.byref(ms), ct.byref(cnt), ct.byref(by))
    if rc:
        raise RuntimeError(f"ptf_profile_read failed ({rc})")
    return ms.value, cnt.value, by.value


def run_profile_case(args):
    """The FP32 batched stepping alone, default launch shapes, for profilers:
    set_c, `warmup` steps, then `steps` steps, in that order and nothing else
    (launch list: set_c 6 launches, then 8 per step after a 2-launch prologue)."""
    import torch
    import __graft_entry__ as g
    if not (g.PKG_DIR / "libptf.so").exists():
        g.build()
    pkg = g.load_package()
    n, B = args.n, args.batch
    u, v = flow_fns()
    kw = dict(nx=n, Lx=2 * np.pi, κ=1e-4, η=1e-4, κh=1e-12, nκh=2, dt=args.dt, stepper="ETDRK4")
    T = np.float64 if args.profile_fp64 else np.float32
    p = pkg.Problem(pkg.GPU(), pkg.TwoDAdvectingFlow(u=u, v=v), T=T, batch=B, **kw)
    p.tuning = dict(branches=1, solves_per_group=0)
    c0 = initial_conditions(n, B, 1234)
    pkg.set_c(p, c0 if B > 1 else c0[0])
    pkg.stepforward(p, args.warmup)
    pkg.stepforward(p, args.steps)
    p.synchronize()
    torch.cuda.synchronize()
    print(json.dumps({"profile_case": True, "n": n, "batch": B, "precision": "f64" if args.profile_fp64 else "f32",
                      "warmup": args.warmup, "steps": args.steps, "tuning": p.tuning}), flush=True)


def run_workloads_only(args):
    """Only the secondary configurations (for instance the full 10,000-request
    served stream: --workloads-only --only served_fp32 --serve-requests 10000),
    printed as one JSON line; not the contract's bench line."""
    import torch
    import __graft_entry__ as g
    if not (g.PKG_DIR / "libptf.so").exists():
        g.build()
    pkg = g.load_package()
    torch.cuda.set_device(0)
    sampler = ClockSampler(torch.cuda.current_device())
    sampler.start()
    w = run_workloads(args, pkg, torch)
    print(json.dumps({"workloads_only": True, "workloads": w, "clocks": sampler.stop()}), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.workloads_only:
        run_workloads_only(args)
    elif args.profile_case:
        run_profile_case(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
