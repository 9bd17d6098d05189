"""Batched and served forms of the TracerAdvectionDiffusion time step.

No single reference counterpart: the reference steps one ``Problem`` at a
time.  :class:`BatchedProblem` steps many independent 2D problems (each with
its own size, diffusivity, dt, clock, step count and flow) together on one
GPU; :class:`Server` adds continuous batching of submitted requests with
admission by device-memory budget and latency statistics.  Both wrap the C
ABI of libptf.so (``ptf_batch_*``, ``ptf_server_*``).
"""
from __future__ import annotations

import ctypes as ct
import math
from dataclasses import dataclass

import numpy as np

from . import _lib as L


@dataclass
class SolveSpec:
    """One solve: grid ``n`` per axis on ``[-L/2, L/2)``, RK4 with ``dt`` for
    ``nsteps`` steps.  ``flow`` is ``"arrays"`` (steady grid arrays passed at
    submission) or ``"cellular"``: ψ = U cos(Kx x + ε sin ω t) cos(Ky y), u = -∂ψ/∂y,
    v = ∂ψ/∂x, evaluated at ``clock.t`` (``time_mode="clock"``, the reference's
    rule) or at each RK4 stage time (``"stage"``)."""
    n: int
    nsteps: int
    dt: float
    kappa: float = 0.0
    eta: float | None = None
    kappah: float = 0.0
    nkappah: int = 0
    L: float = 2 * math.pi
    dim: int = 2
    flow: str = "arrays"
    time_mode: str = "clock"
    U: float = 1.0
    eps: float = 0.0
    omega: float = 0.0
    Kx: int = 1
    Ky: int = 1

    def desc(self) -> L.PtfSolveDesc:
        d = L.PtfSolveDesc()
        L.load().ptf_solve_desc_default(ct.byref(d))
        d.dim, d.n, d.L = self.dim, self.n, self.L
        d.kappa = self.kappa
        d.eta = self.kappa if self.eta is None else self.eta
        d.kappah, d.nkappah = self.kappah, self.nkappah
        d.dt, d.nsteps = self.dt, self.nsteps
        d.flow_kind = {"arrays": L.PTF_FLOW_ARRAYS, "cellular": L.PTF_FLOW_CELLULAR}[self.flow]
        d.time_mode = {"clock": L.PTF_CLOCK_T, "stage": L.PTF_STAGE_T}[self.time_mode]
        d.U, d.eps, d.omega, d.Kx, d.Ky = self.U, self.eps, self.omega, self.Kx, self.Ky
        return d

    @property
    def points(self):
        return self.n ** self.dim


def _f64(a, shape):
    return np.ascontiguousarray(np.broadcast_to(np.asarray(a, dtype=np.float64), shape))


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ct.c_void_p)


_PREC = {np.float64: L.PTF_FP64, np.float32: L.PTF_FP32}


class BatchedProblem:
    """Independent 2D solves stepped together (RK4; per stage one row launch and
    one column launch over all solves' work items -- or one persistent kernel
    with ``persistent=True`` -- steps replayed from a captured CUDA graph)."""

    def __init__(self, T=np.float32, memory_budget=0, slots_per_bucket=0, use_graph=True, max_slots=4096,
                 persistent=False, k0_mode=True):
        lib = L.load()
        cfg = L.PtfBatchConfig()
        lib.ptf_batch_config_default(ct.byref(cfg))
        cfg.precision = _PREC[T]
        cfg.memory_budget = int(memory_budget)
        cfg.slots_per_bucket = int(slots_per_bucket)
        cfg.use_graph = 1 if use_graph else 0
        cfg.max_slots = int(max_slots)
        cfg.persistent = 1 if persistent else 0
        cfg.k0_mode = 1 if k0_mode else 0
        h = ct.c_void_p()
        L.check(lib.ptf_batch_create(ct.byref(cfg), ct.byref(h)), None)
        self._h = h
        self.specs = {}

    def _check(self, rc):
        L.check(rc, self._h, L.load().ptf_batch_last_error)

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            L.load().ptf_batch_destroy(self._h)
            self._h = None

    __del__ = close

    def add(self, spec: SolveSpec, c0, u=None, v=None) -> int:
        shape = (spec.n, spec.n)
        c0 = _f64(c0, shape)
        u = None if u is None else _f64(u, shape)
        v = None if v is None else _f64(v, shape)
        d = spec.desc()
        sid = ct.c_int64()
        self._check(L.load().ptf_batch_add(self._h, ct.byref(d), _ptr(c0), _ptr(u), _ptr(v), ct.byref(sid)))
        self.specs[sid.value] = spec
        return sid.value

    def step(self, nsteps: int = 1):
        self._check(L.load().ptf_batch_step(self._h, int(nsteps)))

    def synchronize(self):
        self._check(L.load().ptf_batch_synchronize(self._h))

    def inject_wait_timeout(self, extra_row_items=1, spin_limit=0):
        """Failure-detection test hook (persistent form): column items wait for
        row items that do not exist until their bounded wait runs out; the next
        ``synchronize`` raises.  Nothing faults on the GPU."""
        self._check(L.load().ptf_batch_inject_wait_timeout(self._h, int(extra_row_items), int(spin_limit)))

    def status(self, sid):
        st, t, act = ct.c_int64(), ct.c_double(), ct.c_int32()
        self._check(L.load().ptf_batch_status(self._h, sid, ct.byref(st), ct.byref(t), ct.byref(act)))
        return st.value, t.value, bool(act.value)

    def get_c(self, sid):
        n = self.specs[sid].n
        out = np.empty((n, n))
        self._check(L.load().ptf_batch_get_c(self._h, sid, _ptr(out)))
        return out

    def remove(self, sid):
        self._check(L.load().ptf_batch_remove(self._h, sid))
        self.specs.pop(sid, None)

    @property
    def stream(self):
        p = ct.c_void_p()
        self._check(L.load().ptf_batch_get_stream(self._h, ct.byref(p)))
        return p.value

    def info(self):
        b, s, k = ct.c_int64(), ct.c_int64(), ct.c_int64()
        self._check(L.load().ptf_batch_info(self._h, ct.byref(b), ct.byref(s), ct.byref(k)))
        return {"device_bytes": b.value, "solves": s.value, "kernel_launches": k.value}


class Server:
    """Continuous-batching request server (worker thread in the library)."""

    def __init__(self, T=np.float32, memory_budget=0, chunk_steps=50, slots_per_bucket=0):
        lib = L.load()
        cfg = L.PtfServerConfig()
        lib.ptf_server_config_default(ct.byref(cfg))
        cfg.precision = _PREC[T]
        cfg.memory_budget = int(memory_budget)
        cfg.chunk_steps = int(chunk_steps)
        cfg.slots_per_bucket = int(slots_per_bucket)
        h = ct.c_void_p()
        L.check(lib.ptf_server_create(ct.byref(cfg), ct.byref(h)), None)
        self._h = h
        self.specs = {}

    def _check(self, rc):
        L.check(rc, self._h, L.load().ptf_server_last_error)

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            L.load().ptf_server_destroy(self._h)
            self._h = None

    __del__ = close

    def submit(self, spec: SolveSpec, c0, u=None, v=None, w=None) -> int:
        shape = (spec.n,) * spec.dim
        arrs = [None if a is None else _f64(a, shape) for a in (c0, u, v, w)]
        d = spec.desc()
        rid = ct.c_int64()
        self._check(L.load().ptf_server_submit(self._h, ct.byref(d), *[_ptr(a) for a in arrs], ct.byref(rid)))
        self.specs[rid.value] = spec
        return rid.value

    def poll(self, rid):
        """(state, field or None); state is "queued", "active", "done" or "failed"."""
        spec = self.specs[rid]
        out = np.empty((spec.n,) * spec.dim)
        st = ct.c_int32()
        self._check(L.load().ptf_server_poll(self._h, rid, ct.byref(st), _ptr(out)))
        name = {0: "queued", 1: "active", 2: "done", 3: "failed"}[st.value]
        return name, (out if name == "done" else None)

    def release(self, rid):
        self._check(L.load().ptf_server_release(self._h, rid))
        self.specs.pop(rid, None)

    def wait_all(self, timeout=600.0):
        self._check(L.load().ptf_server_wait_all(self._h, float(timeout)))

    def stats(self):
        s = L.PtfServerStats()
        self._check(L.load().ptf_server_get_stats(self._h, ct.byref(s)))
        return {f: getattr(s, f) for f, _ in s._fields_}

    def result_info(self, rid):
        """Latency (s) and tracer mass (sum of c, compensated FP64) of the initial
        condition and of the result of a finished request; its mass drift is
        ``mass_end / mass0 - 1``."""
        lat, m0, m1 = ct.c_double(), ct.c_double(), ct.c_double()
        self._check(L.load().ptf_server_result_info(self._h, rid, ct.byref(lat), ct.byref(m0), ct.byref(m1)))
        return {"latency_s": lat.value, "mass0": m0.value, "mass_end": m1.value,
                "mass_drift": (m1.value / m0.value - 1.0) if m0.value else float("nan")}

    def inject_step_failure(self, chunks_from_now=0):
        """Test hook: the chunk of steps that many chunks after the next one
        reports a step failure (host-side; nothing is faulted on the GPU)."""
        self._check(L.load().ptf_server_inject_step_failure(self._h, int(chunks_from_now)))
