"""ctypes binding of libptf.so (the C ABI declared in include/ptf.h).

The library is loaded from this package directory.  There is no fallback:
if the library is missing or no CUDA device is present, the calls raise.
"""
from __future__ import annotations

import ctypes as ct
import os
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libptf.so"
# PTF_ABI_VERSION of include/ptf.h that the structs and signatures below mirror
ABI_VERSION = 4

PTF_OK, PTF_ERR_ARG, PTF_ERR_CUDA, PTF_ERR_STATE, PTF_ERR_UNSUPPORTED, PTF_ERR_MEMORY = 0, 1, 2, 3, 4, 5
PTF_RK4, PTF_ETDRK4, PTF_FILTERED_RK4, PTF_FILTERED_ETDRK4 = 0, 1, 2, 3
PTF_FP64, PTF_FP32 = 0, 1
PTF_CLOCK_T, PTF_STAGE_T = 0, 1
PTF_HOST, PTF_DEVICE = 0, 1


class PtfConfig(ct.Structure):
    _fields_ = [
        ("dim", ct.c_int32), ("nx", ct.c_int32), ("ny", ct.c_int32), ("nz", ct.c_int32),
        ("Lx", ct.c_double), ("Ly", ct.c_double), ("Lz", ct.c_double),
        ("kappa", ct.c_double), ("eta", ct.c_double), ("iota", ct.c_double),
        ("kappah", ct.c_double), ("nkappah", ct.c_int32),
        ("dt", ct.c_double),
        ("stepper", ct.c_int32), ("precision", ct.c_int32), ("time_mode", ct.c_int32),
        ("batch", ct.c_int32), ("k0_mode", ct.c_int32),
    ]


PTF_FLOW_ARRAYS, PTF_FLOW_CELLULAR, PTF_FLOW_ABC = 0, 1, 2


class PtfFlowDesc(ct.Structure):
    _fields_ = [("kind", ct.c_int32), ("U", ct.c_double), ("eps", ct.c_double), ("omega", ct.c_double),
                ("Kx", ct.c_int32), ("Ky", ct.c_int32), ("A", ct.c_double), ("B", ct.c_double), ("C", ct.c_double)]
PTF_REQ_QUEUED, PTF_REQ_ACTIVE, PTF_REQ_DONE, PTF_REQ_FAILED = 0, 1, 2, 3


class PtfSolveDesc(ct.Structure):
    _fields_ = [
        ("dim", ct.c_int32), ("n", ct.c_int32), ("L", ct.c_double),
        ("kappa", ct.c_double), ("eta", ct.c_double), ("kappah", ct.c_double), ("nkappah", ct.c_int32),
        ("dt", ct.c_double), ("nsteps", ct.c_int64),
        ("flow_kind", ct.c_int32), ("time_mode", ct.c_int32),
        ("U", ct.c_double), ("eps", ct.c_double), ("omega", ct.c_double),
        ("Kx", ct.c_int32), ("Ky", ct.c_int32),
    ]


class PtfBatchConfig(ct.Structure):
    _fields_ = [("precision", ct.c_int32), ("memory_budget", ct.c_int64), ("slots_per_bucket", ct.c_int32),
                ("use_graph", ct.c_int32), ("max_slots", ct.c_int32), ("persistent", ct.c_int32),
                ("k0_mode", ct.c_int32)]


class PtfServerConfig(ct.Structure):
    _fields_ = [("precision", ct.c_int32), ("memory_budget", ct.c_int64), ("chunk_steps", ct.c_int32),
                ("slots_per_bucket", ct.c_int32)]


class PtfServerStats(ct.Structure):
    _fields_ = [("completed", ct.c_int64), ("failed", ct.c_int64), ("queued", ct.c_int64), ("active", ct.c_int64),
                ("p50_s", ct.c_double), ("p99_s", ct.c_double), ("mean_s", ct.c_double),
                ("grid_point_steps", ct.c_double), ("wall_s", ct.c_double), ("device_bytes", ct.c_int64),
                ("mass_drift_max_abs", ct.c_double), ("batch_solves", ct.c_int64), ("handles", ct.c_int64),
                ("admit_s", ct.c_double), ("chunk_s", ct.c_double), ("chunks", ct.c_int64)]


class PtfTuning(ct.Structure):
    _fields_ = [("col_lines", ct.c_int32), ("col_lines_y", ct.c_int32), ("row_pairs", ct.c_int32),
                ("branches", ct.c_int32), ("solves_per_group", ct.c_int32), ("row_staged", ct.c_int32),
                ("col_carveout", ct.c_int32), ("ms_per_step", ct.c_double)]


PTF_TUNE_FORCE = 1


class PtfError(RuntimeError):
    """A libptf call returned a non-zero status."""

    def __init__(self, code, msg):
        super().__init__(f"libptf error {code}: {msg}")
        self.code = code


class PtfArgumentError(PtfError, ValueError):
    pass


# name -> (restype, argtypes)
SIGNATURES = {
    "ptf_abi_version": (ct.c_int32, []),
    "ptf_measure_fma_peak": (ct.c_int, [ct.c_int32, ct.POINTER(ct.c_double)]),
    "ptf_config_default": (None, [ct.POINTER(PtfConfig), ct.c_int32]),
    "ptf_create": (ct.c_int, [ct.POINTER(PtfConfig), ct.POINTER(ct.c_void_p)]),
    "ptf_destroy": (None, [ct.c_void_p]),
    "ptf_last_error": (ct.c_char_p, [ct.c_void_p]),
    "ptf_set_flow_arrays": (ct.c_int, [ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_int32]),
    "ptf_set_c": (ct.c_int, [ct.c_void_p, ct.c_void_p, ct.c_int32]),
    "ptf_get_c": (ct.c_int, [ct.c_void_p, ct.c_void_p, ct.c_int32]),
    "ptf_get_sol": (ct.c_int, [ct.c_void_p, ct.c_void_p, ct.c_int32]),
    "ptf_set_sol": (ct.c_int, [ct.c_void_p, ct.c_void_p, ct.c_int32]),
    "ptf_step": (ct.c_int, [ct.c_void_p, ct.c_int64]),
    "ptf_clock": (ct.c_int, [ct.c_void_p, ct.POINTER(ct.c_double), ct.POINTER(ct.c_int64)]),
    "ptf_set_clock": (ct.c_int, [ct.c_void_p, ct.c_double, ct.c_int64]),
    "ptf_calcN": (ct.c_int, [ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_int32]),
    "ptf_synchronize": (ct.c_int, [ct.c_void_p]),
    "ptf_get_stream": (ct.c_int, [ct.c_void_p, ct.POINTER(ct.c_void_p)]),
    "ptf_set_stream": (ct.c_int, [ct.c_void_p, ct.c_void_p]),
    "ptf_device_bytes": (ct.c_int, [ct.c_void_p, ct.POINTER(ct.c_int64)]),
    "ptf_kernel_launches": (ct.c_int, [ct.c_void_p, ct.POINTER(ct.c_int64)]),
    "ptf_calcN2d_noalloc": (ct.c_int, [ct.c_int32, ct.c_int32, ct.c_double, ct.c_double, ct.c_void_p, ct.c_void_p,
                                       ct.c_void_p, ct.c_void_p, ct.c_void_p]),
    "ptf_batch_config_default": (None, [ct.POINTER(PtfBatchConfig)]),
    "ptf_solve_desc_default": (None, [ct.POINTER(PtfSolveDesc)]),
    "ptf_batch_create": (ct.c_int, [ct.POINTER(PtfBatchConfig), ct.POINTER(ct.c_void_p)]),
    "ptf_batch_destroy": (None, [ct.c_void_p]),
    "ptf_batch_last_error": (ct.c_char_p, [ct.c_void_p]),
    "ptf_batch_can_admit": (ct.c_int, [ct.c_void_p, ct.POINTER(PtfSolveDesc)]),
    "ptf_batch_add": (ct.c_int, [ct.c_void_p, ct.POINTER(PtfSolveDesc), ct.c_void_p, ct.c_void_p, ct.c_void_p,
                                 ct.POINTER(ct.c_int64)]),
    "ptf_batch_step": (ct.c_int, [ct.c_void_p, ct.c_int64]),
    "ptf_batch_inject_wait_timeout": (ct.c_int, [ct.c_void_p, ct.c_int32, ct.c_int64]),
    "ptf_batch_synchronize": (ct.c_int, [ct.c_void_p]),
    "ptf_batch_status": (ct.c_int, [ct.c_void_p, ct.c_int64, ct.POINTER(ct.c_int64), ct.POINTER(ct.c_double),
                                    ct.POINTER(ct.c_int32)]),
    "ptf_batch_get_c": (ct.c_int, [ct.c_void_p, ct.c_int64, ct.c_void_p]),
    "ptf_batch_remove": (ct.c_int, [ct.c_void_p, ct.c_int64]),
    "ptf_batch_info": (ct.c_int, [ct.c_void_p, ct.POINTER(ct.c_int64), ct.POINTER(ct.c_int64),
                                  ct.POINTER(ct.c_int64)]),
    "ptf_batch_get_stream": (ct.c_int, [ct.c_void_p, ct.POINTER(ct.c_void_p)]),
    "ptf_server_config_default": (None, [ct.POINTER(PtfServerConfig)]),
    "ptf_server_create": (ct.c_int, [ct.POINTER(PtfServerConfig), ct.POINTER(ct.c_void_p)]),
    "ptf_server_destroy": (None, [ct.c_void_p]),
    "ptf_server_last_error": (ct.c_char_p, [ct.c_void_p]),
    "ptf_server_submit": (ct.c_int, [ct.c_void_p, ct.POINTER(PtfSolveDesc), ct.c_void_p, ct.c_void_p, ct.c_void_p,
                                     ct.c_void_p, ct.POINTER(ct.c_int64)]),
    "ptf_server_poll": (ct.c_int, [ct.c_void_p, ct.c_int64, ct.POINTER(ct.c_int32), ct.c_void_p]),
    "ptf_server_release": (ct.c_int, [ct.c_void_p, ct.c_int64]),
    "ptf_server_wait_all": (ct.c_int, [ct.c_void_p, ct.c_double]),
    "ptf_server_get_stats": (ct.c_int, [ct.c_void_p, ct.POINTER(PtfServerStats)]),
    "ptf_server_result_info": (ct.c_int, [ct.c_void_p, ct.c_int64, ct.POINTER(ct.c_double), ct.POINTER(ct.c_double),
                                          ct.POINTER(ct.c_double)]),
    "ptf_server_inject_step_failure": (ct.c_int, [ct.c_void_p, ct.c_int32]),
    "ptf_set_schedule": (ct.c_int, [ct.c_void_p, ct.c_int32, ct.c_int32, ct.c_int32]),
    "ptf_set_flow_layers": (ct.c_int, [ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_int32]),
    "ptf_set_flow_analytic": (ct.c_int, [ct.c_void_p, ct.POINTER(PtfFlowDesc)]),
    "ptf_get_tuning": (ct.c_int, [ct.c_void_p, ct.POINTER(PtfTuning)]),
    "ptf_set_tuning": (ct.c_int, [ct.c_void_p, ct.POINTER(PtfTuning)]),
    "ptf_autotune": (ct.c_int, [ct.c_void_p, ct.c_int32, ct.c_int32]),
    "ptf_profile": (ct.c_int, [ct.c_void_p, ct.c_int32]),
    "ptf_profile_read": (ct.c_int, [ct.c_void_p, ct.c_int32, ct.POINTER(ct.c_double), ct.POINTER(ct.c_int64),
                                    ct.POINTER(ct.c_double)]),
}

_lib = None


def load(path: os.PathLike | None = None):
    """Load libptf.so (once) and declare the C signatures."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"{p} is missing: build it first (passivetracerflows.jl_gb300/build.py)")
    lib = ct.CDLL(str(p))
    lib.ptf_abi_version.restype = ct.c_int32
    lib.ptf_abi_version.argtypes = []
    got = lib.ptf_abi_version()
    if got != ABI_VERSION:
        raise RuntimeError(f"{p} has ABI version {got}, this binding needs {ABI_VERSION}: rebuild it "
                           "(passivetracerflows.jl_gb300/build.py)")
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def check(rc: int, handle=None, errfn=None):
    if rc == PTF_OK:
        return
    msg = (errfn or load().ptf_last_error)(handle)
    msg = msg.decode() if msg else ""
    if rc == PTF_ERR_ARG:
        raise PtfArgumentError(rc, msg)
    if rc == PTF_ERR_UNSUPPORTED:
        raise NotImplementedError(msg)
    if rc == PTF_ERR_MEMORY:
        raise MemoryError(msg)
    raise PtfError(rc, msg)
