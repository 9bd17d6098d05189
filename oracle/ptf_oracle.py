"""CPU FP64 oracle for the TracerAdvectionDiffusion time step -- TEST INFRASTRUCTURE ONLY.

This module is the checker, never the product.  Only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline / reference legs of
``bench.py`` may import it.  The CUDA product path never calls into it.

It is a plain NumPy/pocketfft restatement of PassiveTracerFlows.jl's
``TracerAdvectionDiffusion`` module together with the FourierFlows.jl 0.10.5
semantics that module relies on (grid, RK4, ETDRK4, clock).  FourierFlows is an
external dependency that the reference does not vendor (``Project.toml:23``);
its behaviour is restated from its published algorithms and pinned by the
reference's own known-answer tests (``test/test_traceradvectiondiffusion.jl``),
which ``tests/test_oracle_kat.py`` runs against this file.

Parity status: RK4 is pinned by the reference's analytic known-answer tests.
ETDRK4 is not exercised by any reference test; its contour-integral
coefficients follow Kassam & Trefethen (2005) with 32 points on a unit circle
("parity unpinned" for ETDRK4 beyond the analytic diffusion limit, where the
ETDRK4 update is exact and is checked in the tests).  In place of a reference
pin, ``tests/test_oracle_etdrk4.py`` checks the coefficients against the
phi-function closed forms in 100-digit arithmetic and the stepper's fourth-order
convergence.

Layout: NumPy C order with x the LAST (fastest) axis, i.e. a 2D field has
shape ``(ny, nx)`` and a 3D field ``(nz, ny, nx)``.  That is byte-for-byte the
reference's column-major ``(nx, ny[, nz])`` layout.  Transforms use
``scipy.fft`` (pocketfft) in FP64 in place of FFTW.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field
from typing import Callable, Optional

import numpy as np
import scipy.fft as sfft

WORKERS = max(1, os.cpu_count() or 1)


def noflow(*args):
    """Zero velocity; ``src/traceradvectiondiffusion.jl:31``."""
    return 0.0


# --------------------------------------------------------------------------
# Grid (FourierFlows OneDGrid/TwoDGrid/ThreeDGrid semantics)
# --------------------------------------------------------------------------
class Grid:
    """Doubly/triply periodic grid on a domain centred at the origin.

    Follows the FourierFlows grid used at ``src/traceradvectiondiffusion.jl:152,177,205``:
    ``x_i = -Lx/2 + i*Lx/nx`` (i = 0..nx-1); ``kr = 2pi/Lx*[0..nx/2]`` (real-FFT
    axis x); ``l, m = 2pi/L*fftfreq`` order; ``Krsq = kr^2 + l^2 (+ m^2)``.
    """

    def __init__(self, dim, nx, Lx, ny=None, Ly=None, nz=None, Lz=None):
        self.dim = dim
        self.nx, self.Lx = int(nx), float(Lx)
        self.ny = int(ny if ny is not None else nx) if dim >= 2 else 1
        self.Ly = float(Ly if Ly is not None else Lx) if dim >= 2 else 0.0
        self.nz = int(nz if nz is not None else nx) if dim >= 3 else 1
        self.Lz = float(Lz if Lz is not None else Lx) if dim >= 3 else 0.0
        self.dx = self.Lx / self.nx
        self.x = -self.Lx / 2 + self.dx * np.arange(self.nx)
        self.nkr = self.nx // 2 + 1
        kr = 2 * np.pi / self.Lx * np.arange(self.nkr)
        if dim == 1:
            self.shape = (self.nx,)
            self.kr = kr
            self.Krsq = kr ** 2
            self.l = self.m = None
        elif dim == 2:
            self.dy = self.Ly / self.ny
            self.y = -self.Ly / 2 + self.dy * np.arange(self.ny)
            self.shape = (self.ny, self.nx)
            self.kr = kr[None, :]
            self.l = (2 * np.pi / self.Ly * np.fft.fftfreq(self.ny, 1.0 / self.ny))[:, None]
            self.m = None
            self.Krsq = self.kr ** 2 + self.l ** 2
        else:
            self.dy = self.Ly / self.ny
            self.dz = self.Lz / self.nz
            self.y = -self.Ly / 2 + self.dy * np.arange(self.ny)
            self.z = -self.Lz / 2 + self.dz * np.arange(self.nz)
            self.shape = (self.nz, self.ny, self.nx)
            self.kr = kr[None, None, :]
            self.l = (2 * np.pi / self.Ly * np.fft.fftfreq(self.ny, 1.0 / self.ny))[None, :, None]
            self.m = (2 * np.pi / self.Lz * np.fft.fftfreq(self.nz, 1.0 / self.nz))[:, None, None]
            self.Krsq = self.kr ** 2 + self.l ** 2 + self.m ** 2
        self.spec_shape = self.shape[:-1] + (self.nkr,)

    def gridpoints(self):
        """Full coordinate arrays (FourierFlows ``gridpoints``), x fastest."""
        if self.dim == 1:
            return (self.x.copy(),)
        if self.dim == 2:
            Y, X = np.meshgrid(self.y, self.x, indexing="ij")
            return X, Y
        Z, Y, X = np.meshgrid(self.z, self.y, self.x, indexing="ij")
        return X, Y, Z

    # rfft along x, complex FFT along the other axes; unnormalised forward,
    # normalised inverse -- ``mul!``/``ldiv!`` with ``grid.rfftplan``.
    def rfft(self, a):
        return sfft.rfftn(np.asarray(a, dtype=np.float64), workers=WORKERS)

    def irfft(self, ah):
        return sfft.irfftn(ah, s=self.shape, workers=WORKERS)


# --------------------------------------------------------------------------
# Flows and parameters
# --------------------------------------------------------------------------
@dataclass
class AdvectingFlow:
    """``OneD/TwoD/ThreeDAdvectingFlow`` (``src/traceradvectiondiffusion.jl:41-106``)."""
    dim: int
    u: Callable = noflow
    v: Callable = noflow
    w: Callable = noflow
    steadyflow: bool = True


def OneDAdvectingFlow(*, u=noflow, steadyflow=True):
    return AdvectingFlow(1, u, noflow, noflow, steadyflow)


def TwoDAdvectingFlow(*, u=noflow, v=noflow, steadyflow=True):
    return AdvectingFlow(2, u, v, noflow, steadyflow)


def ThreeDAdvectingFlow(*, u=noflow, v=noflow, w=noflow, steadyflow=True):
    return AdvectingFlow(3, u, v, w, steadyflow)


def _eval(f, shape, *args):
    return np.broadcast_to(np.asarray(f(*args), dtype=np.float64), shape).copy()


@dataclass
class Params:
    """Steady (``:375-414,426-452``) or time-varying (``:268-348``) parameters.

    Steady flows are evaluated once on the grid (``:437-439``); time-varying
    flows keep the functions and are evaluated at ``clock.t`` inside calcN.
    ``stage_time`` is an extension (not in the reference): evaluate the flow
    at the stage time instead of ``clock.t``.
    """
    kappa: float
    eta: float
    iota: float
    kappah: float
    nkappah: int
    flow: AdvectingFlow
    steady: bool
    ugrid: Optional[tuple] = None
    stage_time: bool = False


def linear_operator(p: Params, g: Grid):
    """``Equation``: ``L = -κ kr² - η l² (- ι m²) - κh Krsq^nκh`` (``:502-554``)."""
    L = -p.kappa * g.kr ** 2
    if g.dim >= 2:
        L = L - p.eta * g.l ** 2
    if g.dim >= 3:
        L = L - p.iota * g.m ** 2
    L = L - p.kappah * g.Krsq ** p.nkappah
    return np.broadcast_to(L, g.spec_shape).astype(np.float64).copy()


def calcN(N_out, sol, t, clock, p: Params, g: Grid):
    """Advective term ``N = rfft(-(u·∇c))``.

    Steady 2D ``src/traceradvectiondiffusion.jl:756-769``, 3D ``:771-786``,
    1D ``:744-754``; time-varying 2D ``:708-723`` (flow at ``clock.t``), 3D
    ``:725-742``, 1D ``:695-706``.
    """
    cx = g.irfft(1j * g.kr * sol)
    if g.dim >= 2:
        cy = g.irfft(1j * g.l * sol)
    if g.dim >= 3:
        cz = g.irfft(1j * g.m * sol)
    if p.steady:
        vel = p.ugrid
    else:
        tf = t if p.stage_time else clock.t
        pts = g.gridpoints()
        fs = (p.flow.u, p.flow.v, p.flow.w)[: g.dim]
        vel = tuple(_eval(f, g.shape, *pts, tf) for f in fs)
    n = -vel[0] * cx
    if g.dim >= 2:
        n = n - vel[1] * cy
    if g.dim >= 3:
        n = n - vel[2] * cz
    N_out[...] = g.rfft(n)


# --------------------------------------------------------------------------
# Time steppers (FourierFlows 0.10.5 RK4 / ETDRK4)
# --------------------------------------------------------------------------
@dataclass
class Clock:
    dt: float
    t: float = 0.0
    step: int = 0


class RK4:
    """Classical RK4 on ``ŝ' = L ŝ + N(ŝ)`` as FourierFlows does it: each RHS is
    ``calcN! + L .* sol``; substeps at ``sol + dt/2 RHS₁``, ``sol + dt/2 RHS₂``,
    ``sol + dt RHS₃``; update ``sol += dt (RHS₁/6 + RHS₂/3 + RHS₃/3 + RHS₄/6)``.
    """

    def __init__(self, L, dt):
        self.L = L

    def step(self, sol, clock, p, g):
        dt, t, L = clock.dt, clock.t, self.L
        R = [np.empty_like(sol) for _ in range(4)]
        calcN(R[0], sol, t, clock, p, g)
        R[0] += L * sol
        s1 = sol + dt / 2 * R[0]
        calcN(R[1], s1, t + dt / 2, clock, p, g)
        R[1] += L * s1
        s1 = sol + dt / 2 * R[1]
        calcN(R[2], s1, t + dt / 2, clock, p, g)
        R[2] += L * s1
        s1 = sol + dt * R[2]
        calcN(R[3], s1, t + dt, clock, p, g)
        R[3] += L * s1
        sol += dt * (R[0] / 6 + R[1] / 3 + R[2] / 3 + R[3] / 6)


NCIRC = 32
RCIRC = 1.0


def etdrk4_coefficients(dt, L, ncirc=NCIRC, rcirc=RCIRC, chunk=1 << 16):
    """ETDRK4 coefficients by the Kassam-Trefethen (2005) contour mean.

    Returns ``(expLdt, expLdt2, ζ, α, β, Γ)`` real arrays of L's shape:
    ``ζ = dt·mean((e^{z/2}-1)/z)``, ``α = dt·mean((-4-z+e^z(4-3z+z²))/z³)``,
    ``β = dt·mean((2+z+e^z(z-2))/z³)``, ``Γ = dt·mean((-4-3z-z²+e^z(4-z))/z³)``
    over ``z = dt·L + rcirc·exp(2πi(j+½)/ncirc)``.
    """
    Lf = np.asarray(L, dtype=np.float64).reshape(-1)
    circ = rcirc * np.exp(2j * np.pi / ncirc * (np.arange(ncirc) + 0.5))
    outs = [np.empty_like(Lf) for _ in range(4)]
    for a in range(0, Lf.size, chunk):
        z = dt * Lf[a:a + chunk, None] + circ[None, :]
        ez = np.exp(z)
        z3 = z ** 3
        outs[0][a:a + chunk] = dt * np.real(np.mean((np.exp(z / 2) - 1) / z, axis=1))
        outs[1][a:a + chunk] = dt * np.real(np.mean((-4 - z + ez * (4 - 3 * z + z * z)) / z3, axis=1))
        outs[2][a:a + chunk] = dt * np.real(np.mean((2 + z + ez * (-2 + z)) / z3, axis=1))
        outs[3][a:a + chunk] = dt * np.real(np.mean((-4 - 3 * z - z * z + ez * (4 - z)) / z3, axis=1))
    shp = np.shape(L)
    return (np.exp(dt * L), np.exp(dt * L / 2)) + tuple(o.reshape(shp) for o in outs)


class ETDRK4:
    """Cox-Matthews ETDRK4 as FourierFlows stores and applies it:
    a = E₂ŝ + ζN(ŝ); b = E₂ŝ + ζN(a); c = E₂a + ζ(2N(b) - N(ŝ));
    ŝ ← Eŝ + αN(ŝ) + 2β(N(a) + N(b)) + ΓN(c).
    """

    def __init__(self, L, dt):
        self.E, self.E2, self.zeta, self.alpha, self.beta, self.gamma = etdrk4_coefficients(dt, L)

    def step(self, sol, clock, p, g):
        dt, t = clock.dt, clock.t
        N1, N2, N3, N4 = (np.empty_like(sol) for _ in range(4))
        calcN(N1, sol, t, clock, p, g)
        s1 = self.E2 * sol + self.zeta * N1
        calcN(N2, s1, t + dt / 2, clock, p, g)
        s2 = self.E2 * sol + self.zeta * N2
        calcN(N3, s2, t + dt / 2, clock, p, g)
        s2 = self.E2 * s1 + self.zeta * (2 * N3 - N1)
        calcN(N4, s2, t + dt, clock, p, g)
        sol[...] = (self.E * sol + self.alpha * N1 + 2 * self.beta * (N2 + N3) + self.gamma * N4)


def makefilter(g: Grid, order=4, innerK=0.65, outerK=1.0, tol=1e-15):
    """FourierFlows' spectral filter (``makefilter``, used by its Filtered
    steppers; FourierFlows is not in the reference tree, so this restates its
    published form -- parity unpinned): ``K = |(kr dx, l dy[, m dz])| / pi``;
    1 for ``K < innerK``, else ``exp(-decay (K - innerK)^order)`` with
    ``decay = -log(tol) / (outerK - innerK)^order``."""
    K2 = (g.kr * g.dx / np.pi) ** 2
    if g.dim >= 2:
        K2 = K2 + (g.l * g.dy / np.pi) ** 2
    if g.dim >= 3:
        K2 = K2 + (g.m * g.dz / np.pi) ** 2
    K = np.broadcast_to(np.sqrt(K2), g.spec_shape)
    decay = -np.log(tol) / (outerK - innerK) ** order
    return np.where(K < innerK, 1.0, np.exp(-decay * np.clip(K - innerK, 0, None) ** order))


class FilteredRK4(RK4):
    """FourierFlows FilteredRK4: an RK4 step, then ``sol .*= filter``."""

    def __init__(self, L, dt, g):
        super().__init__(L, dt)
        self.filter = makefilter(g)

    def step(self, sol, clock, p, g):
        super().step(sol, clock, p, g)
        sol *= self.filter


class FilteredETDRK4(ETDRK4):
    """FourierFlows FilteredETDRK4: an ETDRK4 step, then ``sol .*= filter``."""

    def __init__(self, L, dt, g):
        super().__init__(L, dt)
        self.filter = makefilter(g)

    def step(self, sol, clock, p, g):
        super().step(sol, clock, p, g)
        sol *= self.filter


STEPPERS = {"RK4": RK4, "ETDRK4": ETDRK4, "FilteredRK4": FilteredRK4, "FilteredETDRK4": FilteredETDRK4}


# --------------------------------------------------------------------------
# Problem (the reference API restated)
# --------------------------------------------------------------------------
@dataclass
class Vars:
    c: np.ndarray
    ch: np.ndarray


class Problem:
    """``TracerAdvectionDiffusion.Problem(dev, flow; nx, Lx, ny, Ly, nz, Lz, κ, η, ι, dt, stepper)``
    (``src/traceradvectiondiffusion.jl:143-216``).  ``kappah``/``nkappah`` expose the
    hyperdiffusion reachable in the reference only through the low-level
    ``ConstDiffSteadyFlowParams`` constructor (``test/…:420-423``).
    """

    def __init__(self, flow: AdvectingFlow, *, nx=128, Lx=2 * np.pi, ny=None, Ly=None,
                 nz=None, Lz=None, kappa=0.1, eta=None, iota=None, kappah=0.0, nkappah=0,
                 dt=0.01, stepper="RK4", stage_time=False):
        g = Grid(flow.dim, nx, Lx, ny, Ly, nz, Lz)
        eta = kappa if eta is None else eta
        iota = kappa if iota is None else iota
        p = Params(kappa, eta, iota, kappah, nkappah, flow, flow.steadyflow, stage_time=stage_time)
        if flow.steadyflow:
            pts = g.gridpoints()
            fs = (flow.u, flow.v, flow.w)[: g.dim]
            p.ugrid = tuple(_eval(f, g.shape, *pts) for f in fs)
        self.grid, self.params = g, p
        self.L = linear_operator(p, g)
        self.clock = Clock(dt=float(dt))
        self.sol = np.zeros(g.spec_shape, dtype=np.complex128)
        self.vars = Vars(np.zeros(g.shape), np.zeros(g.spec_shape, dtype=np.complex128))
        if stepper not in STEPPERS:
            raise ValueError(f"unsupported stepper {stepper!r}")
        self.stepper_name = stepper
        if stepper.startswith("Filtered"):
            self.timestepper = STEPPERS[stepper](self.L, float(dt), g)
        else:
            self.timestepper = STEPPERS[stepper](self.L, float(dt))

    def set_flow_arrays(self, *vel):
        """Steady flow given directly as grid arrays (device-array flow input)."""
        self.params.ugrid = tuple(np.asarray(a, dtype=np.float64).reshape(self.grid.shape) for a in vel)
        self.params.steady = True


class MultiLayerProblem:
    """``Problem(MQGprob; κ, η, stepper="FilteredRK4")`` (``:225-250``): one 2D
    tracer per layer with ``L = -κ kr² - η l²`` (``:556-566``), advected by
    the layer's ``u + U_j``, ``v`` (``calcN!``, ``:788-804``).  The layer
    velocities are set with ``set_layer_flows`` before each step (what
    ``calcN!`` reads from ``MQGprob.vars``)."""

    def __init__(self, *, nx, Lx=2 * np.pi, ny=None, Ly=None, nlayers, dt, kappa=0.1, eta=None,
                 stepper="FilteredRK4"):
        self.layers = [Problem(TwoDAdvectingFlow(), nx=nx, Lx=Lx, ny=ny, Ly=Ly, kappa=kappa, eta=eta, dt=dt,
                               stepper=stepper) for _ in range(int(nlayers))]
        self.nlayers = int(nlayers)
        self.grid = self.layers[0].grid
        self.clock = self.layers[0].clock

    def set_layer_flows(self, u, v, U=None):
        """``u_j + U_j``, ``v_j`` per layer (``:794-795``).  ``U``: one value
        per layer, or ``(nlayers, ny)`` -- a zonal flow profile U_j(y), which
        broadcasts along x as GeophysicalFlows' ``(ny, nlayers)`` form does."""
        U = np.zeros(self.nlayers) if U is None else np.asarray(U, dtype=np.float64)
        if U.size == self.nlayers:
            U = U.reshape(self.nlayers, 1, 1)
        else:
            U = U.reshape(self.nlayers, self.grid.ny, 1)
        for j, pr in enumerate(self.layers):
            pr.set_flow_arrays(np.asarray(u[j]) + U[j], np.asarray(v[j]))

    @property
    def sol(self):
        return np.stack([pr.sol for pr in self.layers])

    @property
    def c(self):
        return np.stack([pr.vars.c for pr in self.layers])

    def set_c(self, c):
        """``set_c!`` (``:861-870``): one 2D field repeated over the layers (a
        stack of per-layer fields is taken as it is)."""
        c = np.asarray(c, dtype=np.float64)
        if c.ndim == 2:
            c = np.broadcast_to(c, (self.nlayers,) + c.shape)
        for j, pr in enumerate(self.layers):
            set_c(pr, c[j])

    def stepforward(self, nsteps=1):
        for pr in self.layers:
            stepforward(pr, nsteps)
        self.clock = self.layers[0].clock

    def updatevars(self):
        for pr in self.layers:
            updatevars(pr)


def set_c(prob: Problem, c):
    """``set_c!`` (``:844-852``): ``sol = rfft(c)`` then ``updatevars!``."""
    prob.sol[...] = prob.grid.rfft(np.asarray(c, dtype=np.float64).reshape(prob.grid.shape))
    updatevars(prob)


def updatevars(prob: Problem):
    """``updatevars!`` (``:815-821``): ``ch = sol``; ``c = irfft(ch)``."""
    prob.vars.ch[...] = prob.sol
    prob.vars.c[...] = prob.grid.irfft(prob.vars.ch.copy())


def stepforward(prob: Problem, nsteps: int = 1):
    """FourierFlows ``stepforward!``: stepper update, then ``t += dt``, ``step += 1``."""
    for _ in range(int(nsteps)):
        prob.timestepper.step(prob.sol, prob.clock, prob.params, prob.grid)
        prob.clock.t += prob.clock.dt
        prob.clock.step += 1


def _as_num(a):
    a = np.asarray(a)
    return a.astype(np.complex128) if np.iscomplexobj(a) else a.astype(np.float64)


def rel_l2(a, b):
    """‖a-b‖₂ / ‖b‖₂ (real or complex arrays)."""
    a, b = _as_num(a), _as_num(b)
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


def isapprox(a, b, rtol):
    """Julia ``isapprox`` on arrays: ‖a-b‖ ≤ rtol·max(‖a‖, ‖b‖)."""
    a, b = _as_num(a).ravel(), _as_num(b).ravel()
    return bool(np.linalg.norm(a - b) <= rtol * max(np.linalg.norm(a), np.linalg.norm(b)))
