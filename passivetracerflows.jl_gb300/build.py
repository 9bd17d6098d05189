"""Build recipe for libptf.so (sm_103a): compile each CUDA translation unit
with nvcc in parallel and link them into one shared library beside this file.

Run ``python build.py`` (or call :func:`build`).  Objects go to ``_build/``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
INCLUDE = PKG.parent / "include"
BUILD = PKG / "_build"
LIB = PKG / "libptf.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-I", str(INCLUDE),
                     "--expt-relaxed-constexpr"]


def _nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(p).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libptf.so")
    return p


# Per-(precision, length) instantiation units: one source, many objects.
_SIZES = (16, 32, 64, 128, 256, 512, 1024, 2048, 4096)
INST_SOURCES = {
    "ptf_k2d_inst.cu": [(f"{t}_{n}", [f"-DPTF_T={t}", f"-DPTF_N={n}"]) for t in ("float", "double") for n in _SIZES],
    "ptf_batch_inst.cu": [(f"{t}_m{m}", [f"-DPTF_T={t}", f"-DPTF_MODE={m}"]) for t in ("float", "double")
                          for m in (2, 3, 4, 5)],
    "ptf_k1d_inst.cu": [(f"{t}_{n}", [f"-DPTF_T={t}", f"-DPTF_N={n}"]) for t in ("float", "double") for n in _SIZES],
}


def _units():
    """(source, object, extra defines) for every object of the library."""
    units = []
    for src in sorted(CSRC.glob("*.cu")):
        if src.name in INST_SOURCES:
            for tag, defs in INST_SOURCES[src.name]:
                units.append((src, BUILD / f"{src.stem}_{tag}.o", defs))
        else:
            units.append((src, BUILD / (src.stem + ".o"), []))
    return units


def _deps():
    return sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + sorted(INCLUDE.glob("*.h"))


def _compile(nvcc: str, src: Path, obj: Path, extra) -> None:
    cmd = [nvcc] + NVCC_FLAGS + list(extra) + ["-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stdout}\n{r.stderr}")


def build(force: bool = False, verbose: bool = False, extra=()) -> Path:
    """Compile every ``csrc/*.cu`` and link ``libptf.so``; returns its path."""
    nvcc = _nvcc()
    BUILD.mkdir(exist_ok=True)
    dep_mtime = max((p.stat().st_mtime for p in _deps()), default=0.0)
    jobs = []
    units = _units()
    for src, obj, defs in units:
        stale = force or not obj.exists() or obj.stat().st_mtime < max(src.stat().st_mtime, dep_mtime)
        if stale:
            jobs.append((src, obj, defs))
    workers = max(1, min(len(jobs), os.cpu_count() or 1))
    if jobs:
        # the heavy instantiation units first
        jobs.sort(key=lambda j: (not j[2], "batch" not in j[0].name, -len(str(j[1]))))
        with cf.ThreadPoolExecutor(max_workers=workers) as ex:
            futs = [ex.submit(_compile, nvcc, s, o, list(extra) + d) for s, o, d in jobs]
            for f in futs:
                f.result()
    objs = [str(o) for _, o, _ in units]
    newest = max(Path(o).stat().st_mtime for o in objs)
    if force or jobs or not LIB.exists() or LIB.stat().st_mtime < newest:
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [nvcc] + ARCH + ["-shared", "-o", str(tmp)] + objs + ["-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
