"""The oracle reproduces its committed golden fixtures (CPU)."""
from pathlib import Path

import numpy as np

GOLD = Path(__file__).resolve().parent / "golden"


def _mod():
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", GOLD / "make_golden.py")
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def test_golden_cellular128_rk4(oracle):
    g = np.load(GOLD / "cellular128_rk4.npz")
    d = _mod().cellular128_rk4()
    for k in ("c100", "c2000"):
        assert oracle.rel_l2(d[k], g[k]) <= 1e-13, k
    assert int(g["step"]) == 2000 and abs(float(g["t"]) - 20.0) < 1e-9


def test_golden_cellular128_etdrk4(oracle):
    g = np.load(GOLD / "cellular128_etdrk4.npz")
    d = _mod().cellular128_etdrk4()
    assert oracle.rel_l2(d["c50"], g["c50"]) <= 1e-13


def test_golden_mass_conservation(oracle):
    """Incompressible advection + diffusion conserve Σc up to aliasing round-off."""
    g = np.load(GOLD / "cellular128_rk4.npz")
    m0, m1 = g["c0"].sum(), g["c2000"].sum()
    assert abs(m1 - m0) / abs(m0) < 1e-12


def test_golden_abc32_etdrk4(oracle):
    g = np.load(GOLD / "abc32_etdrk4.npz")
    d = _mod().abc32_etdrk4()
    assert oracle.rel_l2(d["c100"], g["c100"]) <= 1e-13
    m0, m1 = g["c0"].sum(), g["c100"].sum()
    assert abs(m1 - m0) / abs(m0) < 1e-10


def test_golden_line256(oracle):
    g = np.load(GOLD / "line256.npz")
    d = _mod().line256()
    for k in ("c400_RK4", "c400_ETDRK4"):
        assert oracle.rel_l2(d[k], g[k]) <= 1e-13, k
    assert int(g["step"]) == 400
    # RK4 and ETDRK4 agree to their O(dt^4) difference
    assert oracle.rel_l2(g["c400_RK4"], g["c400_ETDRK4"]) <= 1e-9
