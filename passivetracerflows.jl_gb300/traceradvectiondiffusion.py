"""TracerAdvectionDiffusion: the reference module's user-facing API over libptf.so.

Mirrors ``src/traceradvectiondiffusion.jl`` of PassiveTracerFlows.jl:

=============================================  ==========================================
reference (Julia)                              here (Python)
=============================================  ==========================================
``TwoDAdvectingFlow(; u, v, steadyflow)``      ``TwoDAdvectingFlow(u=..., v=..., steadyflow=...)``
``Problem(dev, flow; nx, Lx, ..., κ, dt, ...)`` ``Problem(GPU(), flow, nx=..., κ=..., dt=...)``
``stepforward!(prob, n)``                      ``stepforward(prob, n)``
``set_c!(prob, c)``                            ``set_c(prob, c)``
``updatevars!(prob)``                          ``updatevars(prob)``
``prob.vars.c`` / ``prob.sol`` / ``prob.clock`` same attributes
=============================================  ==========================================

Arrays use NumPy C order with x the last axis, which is byte-identical to the
reference's column-major ``(nx, ny[, nz])`` arrays.  All numerics run in the
CUDA library; this module only converts arguments, evaluates user flow
functions on the grid (as the reference's broadcasts do) and keeps the
``vars.c`` mirror.
"""
from __future__ import annotations

import ctypes as ct
import logging
import math
from dataclasses import dataclass
from typing import Callable

import numpy as np

from . import _lib as L

_log = logging.getLogger("ptf_gb300")

__all__ = [
    "CPU", "GPU", "noflow", "OneDAdvectingFlow", "TwoDAdvectingFlow", "ThreeDAdvectingFlow",
    "OneDGrid", "TwoDGrid", "ThreeDGrid", "gridpoints", "Problem", "set_c", "updatevars", "stepforward",
    "MultiLayerQGFlow", "MultiLayerTracerProblem",
]


class CPU:
    """FourierFlows ``CPU()`` device marker.  This package has no CPU path."""


class GPU:
    """FourierFlows ``GPU()`` device marker (the CUDA device of the library)."""


def noflow(*args):
    """``noflow(args...) = 0.0`` (``src/traceradvectiondiffusion.jl:31``)."""
    return 0.0


@dataclass
class AdvectingFlow:
    """Common base of the advecting-flow containers (``:29``)."""
    u: Callable = noflow
    v: Callable = noflow
    w: Callable = noflow
    steadyflow: bool = True
    dim: int = 2

    def __iter__(self):  # Base.iterate over the fields (``:108-109``)
        fields = {1: (self.u, self.steadyflow), 2: (self.u, self.v, self.steadyflow),
                  3: (self.u, self.v, self.w, self.steadyflow)}[self.dim]
        return iter(fields)

    def __str__(self):  # Base.show (``:110-125``)
        names = ("u", "v", "w")[: self.dim]
        kind = {1: "OneD", 2: "TwoD", 3: "ThreeD"}[self.dim] + "AdvectingFlow"
        lines = [kind] + [f"  ├────────── {n}: {_summary(getattr(self, n))}" for n in names]
        return "\n".join(lines + [f"  └─ steadyflow: {str(self.steadyflow).lower()}"])


def _summary(f):
    return getattr(f, "__name__", type(f).__name__)


def OneDAdvectingFlow(*, u=noflow, steadyflow=True):
    """``OneDAdvectingFlow(; u=noflow, steadyflow=true)`` (``:54``)."""
    return AdvectingFlow(u=u, steadyflow=steadyflow, dim=1)


def TwoDAdvectingFlow(*, u=noflow, v=noflow, steadyflow=True):
    """``TwoDAdvectingFlow(; u=noflow, v=noflow, steadyflow=true)`` (``:79``)."""
    return AdvectingFlow(u=u, v=v, steadyflow=steadyflow, dim=2)


def ThreeDAdvectingFlow(*, u=noflow, v=noflow, w=noflow, steadyflow=True):
    """``ThreeDAdvectingFlow(; u, v, w, steadyflow=true)`` (``:106``)."""
    return AdvectingFlow(u=u, v=v, w=w, steadyflow=steadyflow, dim=3)


class _Grid:
    """Host-side description of the FourierFlows grid the library uses:
    ``x = -L/2 + i L/n``, ``kr = 2π/Lx [0..nx/2]``, ``l, m`` in FFT order."""

    def __init__(self, dim, nx, Lx, ny=None, Ly=None, nz=None, Lz=None):
        self.dim = dim
        self.nx, self.Lx = int(nx), float(Lx)
        self.ny = int(ny if ny is not None else nx) if dim >= 2 else 1
        self.Ly = float(Ly if Ly is not None else Lx) if dim >= 2 else 0.0
        self.nz = int(nz if nz is not None else nx) if dim == 3 else 1
        self.Lz = float(Lz if Lz is not None else Lx) if dim == 3 else 0.0
        self.dx = self.Lx / self.nx
        self.x = -self.Lx / 2 + self.dx * np.arange(self.nx)
        self.nkr = self.nx // 2 + 1
        self.kr = 2 * np.pi / self.Lx * np.arange(self.nkr)
        if dim >= 2:
            self.dy = self.Ly / self.ny
            self.y = -self.Ly / 2 + self.dy * np.arange(self.ny)
            self.l = 2 * np.pi / self.Ly * np.fft.fftfreq(self.ny, 1.0 / self.ny)
        if dim == 1:
            self.shape = (self.nx,)
        elif dim == 3:
            self.dz = self.Lz / self.nz
            self.z = -self.Lz / 2 + self.dz * np.arange(self.nz)
            self.m = 2 * np.pi / self.Lz * np.fft.fftfreq(self.nz, 1.0 / self.nz)
            self.shape = (self.nz, self.ny, self.nx)
        else:
            self.shape = (self.ny, self.nx)
        self.spec_shape = self.shape[:-1] + (self.nkr,)
        self.device = GPU()

    @property
    def Krsq(self):
        if self.dim == 1:
            return self.kr ** 2
        if self.dim == 3:
            return self.kr[None, None, :] ** 2 + self.l[None, :, None] ** 2 + self.m[:, None, None] ** 2
        return self.kr[None, :] ** 2 + self.l[:, None] ** 2


def OneDGrid(dev=None, *, nx, Lx):
    """FourierFlows ``OneDGrid(dev; nx, Lx)`` (host-side description)."""
    return _Grid(1, nx, Lx)


def TwoDGrid(dev=None, *, nx, Lx, ny=None, Ly=None):
    """FourierFlows ``TwoDGrid(dev; nx, Lx, ny, Ly)`` (host-side description)."""
    return _Grid(2, nx, Lx, ny, Ly)


def ThreeDGrid(dev=None, *, nx, Lx, ny=None, Ly=None, nz=None, Lz=None):
    """FourierFlows ``ThreeDGrid(dev; nx, Lx, ny, Ly, nz, Lz)`` (host-side description)."""
    return _Grid(3, nx, Lx, ny, Ly, nz, Lz)


def gridpoints(grid: _Grid):
    """FourierFlows ``gridpoints(grid)``: full coordinate arrays, x fastest (1D: x)."""
    if grid.dim == 1:
        return grid.x.copy()
    if grid.dim == 3:
        Z, Y, X = np.meshgrid(grid.z, grid.y, grid.x, indexing="ij")
        return X, Y, Z
    Y, X = np.meshgrid(grid.y, grid.x, indexing="ij")
    return X, Y


def _pts_tuple(grid):
    p = gridpoints(grid)
    return (p,) if grid.dim == 1 else p


@dataclass
class Params:
    """``ConstDiff{Steady,TimeVarying}FlowParams`` (``:268-452``)."""
    κ: float
    η: float
    ι: float
    κh: float
    nκh: int
    u: object
    v: object
    w: object
    steadyflow: bool


@dataclass
class Vars:
    """``Vars2D/3D`` (``:597-668``): the physical concentration mirror."""
    c: np.ndarray


class Clock:
    """FourierFlows ``Clock``: ``t``, ``dt``, ``step`` read from the library."""

    def __init__(self, prob):
        self._prob = prob

    def _read(self):
        t, s = ct.c_double(), ct.c_int64()
        L.check(L.load().ptf_clock(self._prob._h, ct.byref(t), ct.byref(s)), self._prob._h)
        return t.value, s.value

    @property
    def t(self):
        return self._read()[0]

    @property
    def step(self):
        return self._read()[1]

    @property
    def dt(self):
        return self._prob._cfg.dt


def _kw(kwargs, names, default):
    for n in names:
        if n in kwargs:
            return kwargs.pop(n)
    return default


def _is_device(a):
    return hasattr(a, "is_cuda") and a.is_cuda


def _device_array(a, numel, what):
    """A CUDA tensor handed to the library by pointer: the library reads
    exactly ``numel`` float64 values from it, so anything else is refused."""
    import torch
    if a.dtype != torch.float64 or not a.is_contiguous():
        raise ValueError(f"{what}: device arrays must be contiguous float64 tensors")
    if a.numel() != numel:
        raise ValueError(f"{what}: {a.numel()} values on the device, {numel} expected")
    return a


def _all_host_or_device(arrays, what):
    dev = [_is_device(a) for a in arrays]
    if any(dev) and not all(dev):
        raise ValueError(f"{what}: pass all arrays on the host or all on the device, not a mix")
    return all(dev) and len(dev) > 0


def _eval_on_grid(f, shape, pts, *extra):
    return np.ascontiguousarray(np.broadcast_to(np.asarray(f(*pts, *extra), dtype=np.float64), shape))


class Problem:
    """``TracerAdvectionDiffusion.Problem(dev, advecting_flow; nx=128, Lx=2π, ny=nx,
    Ly=Lx, [nz=nx, Lz=Lx,] κ=0.1, η=κ, [ι=κ,] dt=0.01, stepper="RK4", T=Float64)``
    (``src/traceradvectiondiffusion.jl:165-216``).

    Extensions (keyword-only): ``κh``/``nκh`` (hyperdiffusion, reachable in the
    reference only through ``ConstDiffSteadyFlowParams``), ``batch`` (independent
    solves sharing grid, parameters and flow), ``time_mode`` ("clock" as the
    reference, or "stage").  ``T=np.float32`` selects the FP32 form, in which
    ``k0_fp64`` (default True) carries the conserved (0,0[,0]) mode -- state,
    stage combinations and the mean reported by ``vars.c`` -- in FP64.
    """

    def __new__(cls, dev=None, *args, **kwargs):
        # Problem(MQGprob; ...) (:225-250): a MultiLayerQG problem instead of a
        # device and an advecting flow
        if cls is Problem and _is_multilayer_flow(dev):
            return object.__new__(MultiLayerTracerProblem)
        return object.__new__(cls)

    def __init__(self, dev, advecting_flow: AdvectingFlow, **kwargs):
        if isinstance(dev, CPU) or dev is CPU:
            raise NotImplementedError("this package runs on the GPU only: pass GPU()")
        flow = advecting_flow
        if not isinstance(flow, AdvectingFlow):
            raise TypeError("advecting_flow must be a OneD/TwoD/ThreeDAdvectingFlow")
        dim = flow.dim
        nx = int(kwargs.pop("nx", 128))
        Lx = float(kwargs.pop("Lx", 2 * math.pi))
        ny = int(kwargs.pop("ny", nx))
        Ly = float(kwargs.pop("Ly", Lx))
        nz = int(kwargs.pop("nz", nx))
        Lz = float(kwargs.pop("Lz", Lx))
        κ = float(_kw(kwargs, ("κ", "kappa"), 0.1))
        η = float(_kw(kwargs, ("η", "eta"), κ))
        ι = float(_kw(kwargs, ("ι", "iota"), κ))
        κh = float(_kw(kwargs, ("κh", "kappah"), 0.0))
        nκh = int(_kw(kwargs, ("nκh", "nkappah"), 0))
        dt = float(kwargs.pop("dt", 0.01))
        stepper = kwargs.pop("stepper", "RK4")
        T = kwargs.pop("T", np.float64)
        batch = int(kwargs.pop("batch", 1))
        time_mode = kwargs.pop("time_mode", "clock")
        k0_fp64 = bool(kwargs.pop("k0_fp64", True))
        if kwargs:
            raise TypeError(f"unexpected keyword arguments: {sorted(kwargs)}")
        steppers = {"RK4": L.PTF_RK4, "ETDRK4": L.PTF_ETDRK4, "FilteredRK4": L.PTF_FILTERED_RK4,
                    "FilteredETDRK4": L.PTF_FILTERED_ETDRK4}
        if stepper not in steppers:
            raise ValueError(f"stepper {stepper!r} is not supported (RK4, ETDRK4, FilteredRK4, FilteredETDRK4)")
        if T in (np.float64, float, "Float64"):
            prec = L.PTF_FP64
        elif T in (np.float32, "Float32"):
            prec = L.PTF_FP32
        else:
            raise ValueError("T must be np.float64 or np.float32")
        lib = L.load()
        cfg = L.PtfConfig()
        lib.ptf_config_default(ct.byref(cfg), dim)
        cfg.nx, cfg.ny, cfg.nz = nx, ny, nz
        cfg.Lx, cfg.Ly, cfg.Lz = Lx, Ly, Lz
        cfg.kappa, cfg.eta, cfg.iota = κ, η, ι
        cfg.kappah, cfg.nkappah = κh, nκh
        cfg.dt = dt
        cfg.stepper = steppers[stepper]
        cfg.precision = prec
        cfg.time_mode = {"clock": L.PTF_CLOCK_T, "stage": L.PTF_STAGE_T}[time_mode]
        cfg.batch = batch
        cfg.k0_mode = 1 if k0_fp64 else 0
        h = ct.c_void_p()
        L.check(lib.ptf_create(ct.byref(cfg), ct.byref(h)), None)
        self._h = h
        self._cfg = cfg
        self.grid = _Grid(dim, nx, Lx, ny, Ly, nz, Lz)
        self.batch = batch
        self.stepper = stepper
        self.params = Params(κ, η, ι, κh, nκh, flow.u, flow.v, flow.w, flow.steadyflow)
        self.flow = flow
        shape = ((batch,) if batch > 1 else ()) + self.grid.shape
        self.vars = Vars(np.zeros(shape))
        self.clock = Clock(self)
        if flow.steadyflow:
            pts = _pts_tuple(self.grid)
            comps = (flow.u, flow.v, flow.w)[:dim]
            self.set_flow_arrays(*[_eval_on_grid(f, self.grid.shape, pts) for f in comps])
        else:
            self._flow_t = None

    # -- library plumbing ------------------------------------------------------------
    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                L.load().ptf_destroy(h)
            except Exception:
                pass
            self._h = None

    def set_flow_arrays(self, *vel):
        """Set the flow from grid arrays (host NumPy or torch CUDA tensors)."""
        arrs = []
        ptrs = []
        on_device = _all_host_or_device(vel, "set_flow_arrays")
        where = L.PTF_DEVICE if on_device else L.PTF_HOST
        npts = math.prod(self.grid.shape)
        for a in vel:
            if on_device:
                ptrs.append(ct.c_void_p(_device_array(a, npts, "set_flow_arrays").data_ptr()))
                arrs.append(a)
            else:
                a = np.ascontiguousarray(np.broadcast_to(np.asarray(a, dtype=np.float64), self.grid.shape))
                arrs.append(a)
                ptrs.append(a.ctypes.data_as(ct.c_void_p))
        while len(ptrs) < 3:
            ptrs.append(None)
        L.check(L.load().ptf_set_flow_arrays(self._h, ptrs[0], ptrs[1], ptrs[2], where), self._h)

    def set_flow_analytic(self, kind, **p):
        """A flow given by formula, evaluated on the device (``ptf_set_flow_analytic``):
        ``"cellular"`` (2D; ψ = U cos(Kx x + eps sin(omega t)) cos(Ky y), u = -∂ψ/∂y,
        v = ∂ψ/∂x; re-evaluated at ``clock.t`` before every step when eps and
        omega are non-zero) or ``"abc"`` (3D; A, B, C).  Replaces the flow the
        problem was built with; ``stepforward`` then evaluates nothing on the host."""
        d = L.PtfFlowDesc()
        d.kind = {"cellular": L.PTF_FLOW_CELLULAR, "abc": L.PTF_FLOW_ABC}[kind]
        d.U, d.eps, d.omega = float(p.pop("U", 1.0)), float(p.pop("eps", 0.0)), float(p.pop("omega", 0.0))
        d.Kx, d.Ky = int(p.pop("Kx", 1)), int(p.pop("Ky", 1))
        d.A, d.B, d.C = float(p.pop("A", 1.0)), float(p.pop("B", math.sqrt(2 / 3))), float(p.pop("C", math.sqrt(1 / 3)))
        if p:
            raise TypeError(f"unexpected flow parameters: {sorted(p)}")
        L.check(L.load().ptf_set_flow_analytic(self._h, ct.byref(d)), self._h)
        self._device_flow = True

    def _refresh_flow(self):
        """Time-varying flow at ``clock.t`` (``:715-718``), evaluated once per step."""
        t = self.clock.t
        if self._flow_t == t:
            return
        pts = _pts_tuple(self.grid)
        comps = (self.flow.u, self.flow.v, self.flow.w)[: self.grid.dim]
        self.set_flow_arrays(*[_eval_on_grid(f, self.grid.shape, pts, t) for f in comps])
        self._flow_t = t

    @property
    def sol(self):
        """``prob.sol``: the spectral state, complex ``(ny, nx/2+1)`` (C order)."""
        shape = ((self.batch,) if self.batch > 1 else ()) + self.grid.spec_shape
        out = np.empty(shape, dtype=np.complex128)
        L.check(L.load().ptf_get_sol(self._h, out.ctypes.data_as(ct.c_void_p), L.PTF_HOST), self._h)
        return out

    @sol.setter
    def sol(self, value):
        shape = ((self.batch,) if self.batch > 1 else ()) + self.grid.spec_shape
        a = np.ascontiguousarray(np.broadcast_to(np.asarray(value, dtype=np.complex128), shape))
        L.check(L.load().ptf_set_sol(self._h, a.ctypes.data_as(ct.c_void_p), L.PTF_HOST), self._h)

    def calcN(self, sol):
        """The ``calcN!`` plugin (``:744-786``): ``N = rfft(-(u·∇c))`` for ``sol``."""
        shape = ((self.batch,) if self.batch > 1 else ()) + self.grid.spec_shape
        a = np.ascontiguousarray(np.broadcast_to(np.asarray(sol, dtype=np.complex128), shape))
        out = np.empty(shape, dtype=np.complex128)
        if not self.flow.steadyflow and not getattr(self, "_device_flow", False):
            self._refresh_flow()
        L.check(L.load().ptf_calcN(self._h, a.ctypes.data_as(ct.c_void_p), out.ctypes.data_as(ct.c_void_p),
                                   L.PTF_HOST), self._h)
        return out

    def save_state(self, path):
        """Checkpoint: ``sol`` (FP64, including the FP64 k = 0 mode of FP32
        problems) and the clock, to a NumPy ``.npz`` -- what the reference's
        JLD2 output records of a solve (``saveoutput``; the examples save
        ``sol`` and ``clock.t``).  ``load_state`` resumes bit-identically."""
        t, step = self.clock._read()
        cfg = self._cfg
        with open(path, "wb") as f:  # exactly at ``path`` (np.savez would append ".npz")
            np.savez(f, sol=self.sol, t=t, step=step, dim=cfg.dim, nx=cfg.nx, ny=cfg.ny, nz=cfg.nz,
                     batch=cfg.batch, dt=cfg.dt, stepper=cfg.stepper, precision=cfg.precision,
                     **{k: getattr(cfg, k) for k in self._PHYSICS_KEYS})

    # domain and diffusivities a checkpoint must share with the problem it resumes
    _PHYSICS_KEYS = ("Lx", "Ly", "Lz", "kappa", "eta", "iota", "kappah", "nkappah")

    def load_state(self, path):
        """Resume from ``save_state``: the grid, batch, dt, stepper,
        precision, domain lengths and diffusivities must match this problem
        (a checkpoint of other physics is refused, not continued)."""
        with np.load(path) as z:
            cfg = self._cfg
            for k in ("dim", "nx", "ny", "nz", "batch", "stepper", "precision"):
                if int(z[k]) != int(getattr(cfg, k)):
                    raise ValueError(f"checkpoint {k}={int(z[k])} does not match this problem ({getattr(cfg, k)})")
            if float(z["dt"]) != cfg.dt:
                raise ValueError("checkpoint dt does not match this problem")
            for k in self._PHYSICS_KEYS:
                if k not in z.files:
                    raise ValueError(f"checkpoint has no {k}: written by an older version, refused")
                if float(z[k]) != float(getattr(cfg, k)):
                    raise ValueError(f"checkpoint {k}={float(z[k])} does not match this problem ({getattr(cfg, k)})")
            self.sol = z["sol"]
            L.check(L.load().ptf_set_clock(self._h, float(z["t"]), int(z["step"])), self._h)
        if not self.flow.steadyflow and not getattr(self, "_device_flow", False):
            self._flow_t = None

    def set_schedule(self, solves_per_group=0, branches=1, use_graph=True):
        """Step a batch in groups of solves (0: whole batch, or batch/branches),
        dealt to `branches` concurrent stream branches, replaying steps from a
        captured CUDA graph; results do not depend on the schedule."""
        L.check(L.load().ptf_set_schedule(self._h, int(solves_per_group), int(branches), 1 if use_graph else 0),
                self._h)

    _TUNING_FIELDS = ("col_lines", "col_lines_y", "row_pairs", "branches", "solves_per_group", "row_staged",
                      "col_carveout", "ms_per_step")

    @property
    def tuning(self):
        """Launch shapes of this problem (columns / row pairs per block,
        branches, staged row pass) and the tuned ms per step (0: untuned)."""
        t = L.PtfTuning()
        L.check(L.load().ptf_get_tuning(self._h, ct.byref(t)), self._h)
        return {k: getattr(t, k) for k in self._TUNING_FIELDS}

    @tuning.setter
    def tuning(self, value):
        t = L.PtfTuning()
        L.check(L.load().ptf_get_tuning(self._h, ct.byref(t)), self._h)
        for k, v in dict(value).items():
            if k not in self._TUNING_FIELDS:
                raise KeyError(k)
            setattr(t, k, v)
        L.check(L.load().ptf_set_tuning(self._h, ct.byref(t)), self._h)

    def autotune(self, trial_steps=4, force=False):
        """Time candidate launch shapes on this problem (state saved and
        restored) and keep the fastest; cached per shape for the process."""
        L.check(L.load().ptf_autotune(self._h, int(trial_steps), L.PTF_TUNE_FORCE if force else 0), self._h)
        return self.tuning

    def synchronize(self):
        L.check(L.load().ptf_synchronize(self._h), self._h)

    @property
    def stream(self):
        p = ct.c_void_p()
        L.check(L.load().ptf_get_stream(self._h, ct.byref(p)), self._h)
        return p.value

    @property
    def device_bytes(self):
        b = ct.c_int64()
        L.check(L.load().ptf_device_bytes(self._h, ct.byref(b)), self._h)
        return b.value

    @property
    def kernel_launches(self):
        b = ct.c_int64()
        L.check(L.load().ptf_kernel_launches(self._h, ct.byref(b)), self._h)
        return b.value


def set_c(prob: Problem, c):
    """``set_c!(prob, c)`` (``:844-852, :872``): ``sol = rfft(c)``, then ``updatevars!``."""
    if _is_device(c):
        npts = math.prod(prob.grid.shape)
        if prob.batch > 1 and c.numel() == npts:
            # one field for every solve of the batch (for a MultiLayerQG
            # problem: every layer, as set_c! repeats c, :861-870)
            c = c.reshape(prob.grid.shape).expand((prob.batch,) + prob.grid.shape).contiguous()
        c = _device_array(c, prob.batch * npts, "set_c")
        L.check(L.load().ptf_set_c(prob._h, ct.c_void_p(c.data_ptr()), L.PTF_DEVICE), prob._h)
    else:
        shape = ((prob.batch,) if prob.batch > 1 else ()) + prob.grid.shape
        a = np.ascontiguousarray(np.broadcast_to(np.asarray(c, dtype=np.float64), shape))
        L.check(L.load().ptf_set_c(prob._h, a.ctypes.data_as(ct.c_void_p), L.PTF_HOST), prob._h)
    updatevars(prob)


def updatevars(prob: Problem):
    """``updatevars!(prob)`` (``:815-821, :837``): ``vars.c = irfft(sol)``."""
    out = prob.vars.c
    L.check(L.load().ptf_get_c(prob._h, out.ctypes.data_as(ct.c_void_p), L.PTF_HOST), prob._h)


def stepforward(prob: Problem, nsteps: int = 1):
    """FourierFlows ``stepforward!(prob, nsteps)``: ``nsteps`` stepper updates,
    each followed by ``clock.t += dt`` and ``clock.step += 1``.  A time-varying
    flow is re-evaluated at ``clock.t`` before every step, as the reference's
    ``calcN!`` does for all four stages of a step (``:715-718``)."""
    nsteps = int(nsteps)
    if nsteps < 0:
        raise ValueError("nsteps must be non-negative")
    lib = L.load()
    if prob.flow.steadyflow or getattr(prob, "_device_flow", False):
        L.check(lib.ptf_step(prob._h, nsteps), prob._h)
        return
    for _ in range(nsteps):
        prob._refresh_flow()
        L.check(lib.ptf_step(prob._h, 1), prob._h)


# ---------------------------------------------------------------------------
# MultiLayerQG-coupled tracer (src/traceradvectiondiffusion.jl:225-250,
# :455-500, :556-566, :788-804)
# ---------------------------------------------------------------------------
def _is_multilayer_flow(obj):
    return obj is not None and hasattr(obj, "vars") and hasattr(obj, "params") and \
        hasattr(obj.params, "nlayers") and hasattr(obj, "grid") and hasattr(obj, "clock")


def _layer_mean_flow(U, nl, ny):
    """``MQGprob.params.U`` split into what ``ptf_set_flow_layers`` takes: one
    imposed zonal flow per layer (``U_j``), or -- GeophysicalFlows also takes
    a ``(ny, nlayers)`` matrix -- a profile per layer ``U_j(y)``, returned as
    an ``(nl, ny, 1)`` array to add to ``u`` (``calcN!`` adds ``params.U``
    to ``vars.u`` by broadcasting, ``:794``).  Returns ``(per_layer, profile)``
    with one of the two ``None``."""
    U = np.asarray(0.0 if U is None else U, dtype=np.float64)
    if U.size == 1:
        return np.full(nl, float(U.reshape(-1)[0])), None
    if U.size == nl:
        return U.reshape(nl), None
    if U.size == nl * ny:
        return None, U.reshape(nl, ny, 1)
    raise ValueError(f"params.U has {U.size} values: expected 1, nlayers ({nl}) or nlayers x ny ({nl * ny})")


class MultiLayerQGFlow:
    """What the tracer needs of a ``GeophysicalFlows.MultiLayerQG`` problem:
    ``grid`` (nx, Lx, ny, Ly), ``params.nlayers``, ``params.U`` (each layer's
    imposed mean flow), ``clock.dt`` and ``vars.u``, ``vars.v`` (layer
    velocities, ``(nlayers, ny, nx)``, NumPy or contiguous CUDA float64
    tensors).  The QG model itself is not part of this package: the caller
    advances it and updates ``vars``; ``step_until`` (optional) is called for
    ``tracer_release_time > 0``."""

    class _Params:
        def __init__(self, nlayers, U):
            self.nlayers = int(nlayers)
            # one value per layer, or (nlayers, ny): a profile U_j(y) per layer
            self.U = np.zeros(self.nlayers) if U is None else np.asarray(U, dtype=np.float64)

    class _Vars:
        def __init__(self, u, v):
            self.u, self.v = u, v

    class _Clock:
        def __init__(self, dt):
            self.dt, self.t, self.step = float(dt), 0.0, 0

    def __init__(self, *, nx, Lx=2 * math.pi, ny=None, Ly=None, nlayers, dt, U=None, u=None, v=None,
                 step_until=None):
        self.grid = _Grid(2, nx, Lx, ny, Ly)
        self.params = self._Params(nlayers, U)
        shape = (self.params.nlayers,) + self.grid.shape
        self.vars = self._Vars(np.zeros(shape) if u is None else u, np.zeros(shape) if v is None else v)
        self.clock = self._Clock(dt)
        self._step_until = step_until

    def step_until(self, t):
        if self._step_until is None:
            raise NotImplementedError("this MultiLayerQG stand-in cannot advance itself: pass step_until")
        self._step_until(self, t)


class MultiLayerTracerProblem(Problem):
    """``TracerAdvectionDiffusion.Problem(MQGprob; κ=0.1, η=κ, stepper="FilteredRK4",
    tracer_release_time=0)`` (``:225-250``): one tracer per layer, advected by
    that layer's velocity plus its mean flow ``U`` (``calcN!``, ``:788-804``),
    with ``L = -κ kr² - η l²`` (``:556-566``) and the MultiLayerQG problem's
    grid and ``dt``.  The layers are the solves of one batched handle; the
    layer velocities are read from ``MQGprob.vars`` before every step, as
    ``calcN!`` reads them.  Extension: ``T=np.float32``."""

    def __init__(self, MQGprob, κ=0.1, η=None, stepper="FilteredRK4", tracer_release_time=0, T=np.float64, **kw):
        κ = float(kw.pop("kappa", κ))
        η = κ if η is None else float(η)
        η = float(kw.pop("eta", η))
        if kw:
            raise TypeError(f"unexpected keyword arguments: {sorted(kw)}")
        if tracer_release_time < 0:
            raise ValueError("tracer_release_time must be non-negative!")
        if tracer_release_time > 0:
            _log.info("Stepping the flow forward until t = tracer_release_time = %s", tracer_release_time)
            MQGprob.step_until(tracer_release_time)
        self.MQGprob = MQGprob
        g = MQGprob.grid
        nl = int(MQGprob.params.nlayers)
        flow = AdvectingFlow(steadyflow=False, dim=2)
        super().__init__(GPU(), flow, nx=g.nx, Lx=g.Lx, ny=g.ny, Ly=g.Ly, κ=κ, η=η, dt=MQGprob.clock.dt,
                         stepper=stepper, T=T, batch=nl)
        self.nlayers = nl
        self.tracer_release_time = float(tracer_release_time)
        if nl == 1:
            self.vars = Vars(np.zeros((1,) + self.grid.shape))
        self._refresh_flow()

    def _refresh_flow(self):
        """``u = MQGprob.vars.u + MQGprob.params.U``, ``v = MQGprob.vars.v`` (``:794-795``)."""
        mq = self.MQGprob
        U, Uy = _layer_mean_flow(getattr(mq.params, "U", None), self.nlayers, self.grid.ny)
        shape = (self.nlayers,) + self.grid.shape
        ptrs, keep = [], []
        on_device = _all_host_or_device((mq.vars.u, mq.vars.v), "MQGprob.vars.u, v")
        where = L.PTF_DEVICE if on_device else L.PTF_HOST
        u = mq.vars.u
        if Uy is not None:  # a y profile is added to u here; the per-layer constants are then zero
            if on_device:
                import torch
                u = (_device_array(u, math.prod(shape), "MQGprob.vars.u") +
                     torch.as_tensor(Uy, dtype=torch.float64, device=u.device)).contiguous()
            else:
                u = np.broadcast_to(np.asarray(u, dtype=np.float64), shape) + Uy
            U = np.zeros(self.nlayers)
        for a in (u, mq.vars.v):
            if on_device:
                ptrs.append(ct.c_void_p(_device_array(a, math.prod(shape), "MQGprob.vars.u, v").data_ptr()))
                keep.append(a)
            else:
                a = np.ascontiguousarray(np.broadcast_to(np.asarray(a, dtype=np.float64), shape))
                keep.append(a)
                ptrs.append(a.ctypes.data_as(ct.c_void_p))
        Uc = np.ascontiguousarray(U)
        L.check(L.load().ptf_set_flow_layers(self._h, ptrs[0], ptrs[1], Uc.ctypes.data_as(ct.c_void_p), where),
                self._h)
