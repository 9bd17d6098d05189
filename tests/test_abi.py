"""The C ABI library loads, exports every symbol include/ptf.h declares, and
validates arguments before touching the GPU (CPU-only checks)."""
import ctypes as ct
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        src = h.read_text()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names.update(re.findall(r"\b(ptf_[A-Za-z0-9_]+)\s*\(", src))
    return sorted(names)


def test_header_declares_api():
    names = declared_symbols()
    for must in ("ptf_create", "ptf_destroy", "ptf_step", "ptf_set_c", "ptf_get_c", "ptf_get_sol",
                 "ptf_set_flow_arrays", "ptf_calcN", "ptf_clock", "ptf_last_error"):
        assert must in names


def test_library_exports_all_declared(built_lib):
    lib = ct.CDLL(str(built_lib))
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header(pkg):
    from ptf_gb300 import _lib
    missing = [n for n in declared_symbols() if n not in _lib.SIGNATURES]
    assert not missing, missing


def test_binding_abi_version_matches_header_and_library(pkg):
    """The Python binding refuses a library of another ABI version; the
    version it expects is the header's, and the built library reports it."""
    from ptf_gb300 import _lib
    m = re.search(r"#define\s+PTF_ABI_VERSION\s+(\d+)", (ROOT / "include" / "ptf.h").read_text())
    assert m and int(m.group(1)) == _lib.ABI_VERSION
    assert _lib.load().ptf_abi_version() == _lib.ABI_VERSION


def _cfg(pkg, **kw):
    from ptf_gb300 import _lib as L
    lib = L.load()
    c = L.PtfConfig()
    lib.ptf_config_default(ct.byref(c), kw.pop("dim", 2))
    for k, v in kw.items():
        setattr(c, k, v)
    return lib, c


def test_config_defaults_match_reference(pkg):
    lib, c = _cfg(pkg)
    # Problem(dev, flow; nx=128, Lx=2π, κ=0.1, dt=0.01, stepper="RK4") (:165-175)
    assert (c.nx, c.ny) == (128, 128)
    assert abs(c.Lx - 6.283185307179586) < 1e-15 and c.kappa == 0.1 and c.eta == 0.1 and c.dt == 0.01
    assert c.stepper == 0 and c.batch == 1
    assert lib.ptf_abi_version() == 4


@pytest.mark.parametrize("field,value,msg", [
    ("nx", 100, "powers of two"), ("nx", 8192, "powers of two"), ("ny", 8, "powers of two"),
    ("dt", 0.0, "dt"), ("dt", float("nan"), "dt"), ("stepper", 7, "stepper"), ("precision", 3, "precision"),
    ("batch", 0, "batch"), ("Lx", -1.0, "domain"), ("nkappah", -1, "nkappah"),
])
def test_create_rejects_bad_arguments(pkg, field, value, msg):
    from ptf_gb300 import _lib as L
    lib, c = _cfg(pkg, **{field: value})
    h = ct.c_void_p()
    rc = lib.ptf_create(ct.byref(c), ct.byref(h))
    assert rc == L.PTF_ERR_ARG
    assert not h.value
    assert msg in lib.ptf_last_error(None).decode()


@pytest.mark.parametrize("dim", [0, 4])
def test_create_rejects_bad_dimension(pkg, dim):
    from ptf_gb300 import _lib as L
    lib, c = _cfg(pkg, dim=dim)
    h = ct.c_void_p()
    assert lib.ptf_create(ct.byref(c), ct.byref(h)) == L.PTF_ERR_ARG
    assert "dim must be 1, 2 or 3" in lib.ptf_last_error(None).decode()


def test_create_1d_ignores_ny_nz(pkg):
    """1D problems validate nx and Lx only (ny, nz, Ly, Lz are ignored): with no
    GPU here the call gets past argument checking and fails at the device."""
    from ptf_gb300 import _lib as L
    lib, c = _cfg(pkg, dim=1, ny=3, nz=5, Ly=-1.0)
    h = ct.c_void_p()
    rc = lib.ptf_create(ct.byref(c), ct.byref(h))
    assert rc != L.PTF_ERR_ARG


def test_null_handle_calls_fail_cleanly(pkg):
    from ptf_gb300 import _lib as L
    lib = L.load()
    assert lib.ptf_step(None, 1) == L.PTF_ERR_ARG
    assert lib.ptf_set_c(None, None, 0) == L.PTF_ERR_ARG
    assert lib.ptf_synchronize(None) == L.PTF_ERR_ARG
    lib.ptf_destroy(None)


@pytest.mark.parametrize("field,value", [("precision", 7), ("memory_budget", -1), ("slots_per_bucket", -2),
                                         ("max_slots", 0)])
def test_batch_create_rejects_bad_config(pkg, field, value):
    from ptf_gb300 import _lib as L
    lib = L.load()
    c = L.PtfBatchConfig()
    lib.ptf_batch_config_default(ct.byref(c))
    setattr(c, field, value)
    b = ct.c_void_p()
    assert lib.ptf_batch_create(ct.byref(c), ct.byref(b)) == L.PTF_ERR_ARG
    assert not b.value and lib.ptf_batch_last_error(None)


@pytest.mark.parametrize("field,value", [("chunk_steps", -1), ("memory_budget", -5), ("precision", 3)])
def test_server_create_rejects_bad_config(pkg, field, value):
    from ptf_gb300 import _lib as L
    lib = L.load()
    c = L.PtfServerConfig()
    lib.ptf_server_config_default(ct.byref(c))
    setattr(c, field, value)
    s = ct.c_void_p()
    assert lib.ptf_server_create(ct.byref(c), ct.byref(s)) == L.PTF_ERR_ARG
    assert not s.value


def test_batch_and_server_null_calls_fail_cleanly(pkg):
    from ptf_gb300 import _lib as L
    lib = L.load()
    assert lib.ptf_batch_step(None, 1) == L.PTF_ERR_ARG
    assert lib.ptf_batch_synchronize(None) == L.PTF_ERR_ARG
    assert lib.ptf_server_wait_all(None, 0.1) == L.PTF_ERR_ARG
    lib.ptf_batch_destroy(None)
    lib.ptf_server_destroy(None)


def test_noalloc_rejects_bad_arguments_before_the_device(pkg):
    """ptf_calcN2d_noalloc checks sizes, lengths, pointers and the fixed
    scratch's capacity before any CUDA call (the pointers are never read)."""
    from ptf_gb300 import _lib as L
    lib = L.load()
    fake = ct.c_void_p(16)  # never dereferenced: every case fails before the device
    cases = [((100, 64, 1.0, 1.0, fake), L.PTF_ERR_ARG), ((64, 64, -1.0, 1.0, fake), L.PTF_ERR_ARG),
             ((64, 64, 1.0, 1.0, None), L.PTF_ERR_ARG), ((1024, 1024, 1.0, 1.0, fake), L.PTF_ERR_MEMORY)]
    for (nx, ny, Lx, Ly, p), want in cases:
        assert lib.ptf_calcN2d_noalloc(nx, ny, Lx, Ly, p, fake, fake, fake, None) == want
    assert "1024x1024 does not" in lib.ptf_last_error(None).decode()
