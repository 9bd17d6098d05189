"""Snapshot output of a solve: FourierFlows' ``Output`` / ``saveproblem`` /
``saveoutput`` workflow, as the reference's examples use it
(``examples/onedim_gaussiandiffusion.jl:74-88``,
``examples/turbulent_advection-diffusion.jl:126-142``)::

    out = Output(prob, "advection-diffusion.jld2", ("concentration", get_concentration))
    saveproblem(out)
    while prob.clock.step <= nsteps:
        if prob.clock.step % 50 == 0:
            saveoutput(out)
        stepforward(prob)
    f = jldopen(out.path)
    steps = sorted(int(k) for k in f["snapshots/t"].keys())
    c = [f[f"snapshots/concentration/{i}"] for i in steps]

File format.  The reference writes JLD2, an HDF5 file.  Neither JLD2 nor an
HDF5 library is available to this package (``h5py`` is not installed on the
machines it targets), so the same group layout is written as a NumPy ``.npz``
archive (a zip of ``.npy`` members) whose member names are the JLD2 paths:
``grid/nx``, ``grid/Lx``, ``grid/x``, ..., ``params/κ``, ..., ``eqn/L``,
``clock/dt``, ``snapshots/t/<step>``, ``snapshots/<field>/<step>``.  Each
``saveoutput`` appends its members to the archive without rewriting it.
``jldopen`` reads it back with the same paths (a path to a group gives the
group, whose ``keys()`` are its children, as in JLD2).  ``numpy.load`` also
opens the file directly (member ``"snapshots/t/50"`` and so on).

As in FourierFlows, an existing file is never overwritten: ``Output`` picks
the first free name ``<stem>_1<ext>``, ``<stem>_2<ext>``, ....
"""
from __future__ import annotations

import os
import zipfile
from pathlib import Path

import numpy as np

__all__ = ["Output", "saveproblem", "saveoutput", "jldopen", "get_sol", "get_concentration"]


def get_sol(prob):
    """The default field of an ``Output``: the spectral state ``prob.sol``."""
    return prob.sol


def get_concentration(prob):
    """``vars.c`` after ``updatevars`` (the examples' ``get_concentration``)."""
    from .traceradvectiondiffusion import updatevars
    updatevars(prob)
    return prob.vars.c


def _uniquepath(path: Path) -> Path:
    if not path.exists():
        return path
    stem, ext = path.stem, path.suffix
    k = 1
    while True:
        cand = path.with_name(f"{stem}_{k}{ext}")
        if not cand.exists():
            return cand
        k += 1


class Output:
    """``Output(prob, path, (name, fn), ...)``: snapshots of ``fn(prob)`` under
    ``snapshots/<name>/<step>`` (default field: ``("sol", get_sol)``)."""

    def __init__(self, prob, path, *fields):
        self.prob = prob
        self.path = _uniquepath(Path(os.fspath(path)))
        self.fields = list(fields) if fields else [("sol", get_sol)]
        for f in self.fields:
            if not (isinstance(f, tuple) and len(f) == 2 and isinstance(f[0], str) and callable(f[1])):
                raise TypeError("each field is a (name, function of the problem) pair")
        zipfile.ZipFile(self.path, "w").close()  # the file exists from here on

    def _write(self, members):
        with zipfile.ZipFile(self.path, "a", compression=zipfile.ZIP_STORED) as z:
            names = set(z.namelist())
            for name, value in members.items():
                member = name + ".npy"
                if member in names:
                    raise ValueError(f"{self.path} already holds {name}")
                with z.open(member, "w", force_zip64=True) as f:
                    np.lib.format.write_array(f, np.asarray(value), allow_pickle=False)


def _problem_members(prob):
    g = prob.grid
    cfg = prob._cfg
    m = {"grid/nx": g.nx, "grid/Lx": g.Lx, "grid/dx": g.dx, "grid/x": g.x, "grid/kr": g.kr}
    if g.dim >= 2:
        m.update({"grid/ny": g.ny, "grid/Ly": g.Ly, "grid/dy": g.dy, "grid/y": g.y, "grid/l": g.l})
    if g.dim == 3:
        m.update({"grid/nz": g.nz, "grid/Lz": g.Lz, "grid/dz": g.dz, "grid/z": g.z, "grid/m": g.m})
    m.update({"params/κ": cfg.kappa, "params/κh": cfg.kappah, "params/nκh": cfg.nkappah})
    if g.dim >= 2:
        m["params/η"] = cfg.eta
    if g.dim == 3:
        m["params/ι"] = cfg.iota
    # L = -κ kr^2 - η l^2 [- ι m^2] - κh |k|^(2 nκh), the Equation's linear operator
    # (src/traceradvectiondiffusion.jl:538-554), on the half spectrum
    if g.dim == 1:
        L = -cfg.kappa * g.kr ** 2
    elif g.dim == 2:
        L = -cfg.kappa * g.kr[None, :] ** 2 - cfg.eta * g.l[:, None] ** 2
    else:
        L = (-cfg.kappa * g.kr[None, None, :] ** 2 - cfg.eta * g.l[None, :, None] ** 2
             - cfg.iota * g.m[:, None, None] ** 2)
    L = L - cfg.kappah * g.Krsq ** cfg.nkappah
    m["eqn/L"] = L
    m["clock/dt"] = cfg.dt
    return m


def saveproblem(out: Output):
    """Grid, parameters, linear operator and time step of the problem."""
    out._write(_problem_members(out.prob))


def saveoutput(out: Output):
    """One snapshot at the current step: ``snapshots/t/<step>`` and every field."""
    step, t = out.prob.clock.step, out.prob.clock.t
    members = {f"snapshots/t/{step}": t}
    for name, fn in out.fields:
        members[f"snapshots/{name}/{step}"] = np.array(fn(out.prob), copy=True)
    out._write(members)


class _Group:
    def __init__(self, file, prefix):
        self._file, self._prefix = file, prefix

    def keys(self):
        p = self._prefix + "/"
        return sorted({k[len(p):].split("/")[0] for k in self._file._names if k.startswith(p)})

    def __getitem__(self, key):
        return self._file[f"{self._prefix}/{key}"]

    def __contains__(self, key):
        return key in self.keys()


class _File:
    def __init__(self, path):
        self._z = np.load(path, allow_pickle=False)
        self._names = list(self._z.files)

    def __getitem__(self, key):
        key = key.strip("/")
        if key in self._names:
            a = self._z[key]
            return a.item() if a.ndim == 0 else a
        if any(n.startswith(key + "/") for n in self._names):
            return _Group(self, key)
        raise KeyError(key)

    def keys(self):
        return sorted({n.split("/")[0] for n in self._names})

    def close(self):
        self._z.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def jldopen(path):
    """Open an ``Output`` file for reading with JLD2-style paths."""
    return _File(os.fspath(path))
