"""The ctypes mirrors of the C ABI's structs (passivetracerflows.jl_gb300/_lib.py)
have the layout include/ptf.h gives them: a small C program compiled with the
host compiler prints each struct's size and every field's offset, and the
ctypes classes must agree field by field (a mismatch would make the library
read or write past what the caller passed).  No GPU needed."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]

STRUCTS = {
    "ptf_config": "PtfConfig",
    "ptf_flow_desc": "PtfFlowDesc",
    "ptf_tuning": "PtfTuning",
    "ptf_solve_desc": "PtfSolveDesc",
    "ptf_batch_config": "PtfBatchConfig",
    "ptf_server_config": "PtfServerConfig",
    "ptf_server_stats": "PtfServerStats",
}


def test_ctypes_structs_match_the_header(tmp_path):
    import importlib.util
    import sys

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    spec = importlib.util.spec_from_file_location("ptf_lib_layout", ROOT / "passivetracerflows.jl_gb300" / "_lib.py")
    lib = importlib.util.module_from_spec(spec)
    sys.modules["ptf_lib_layout"] = lib
    spec.loader.exec_module(lib)
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "ptf.h"', "int main(void) {"]
    for cname, pyname in STRUCTS.items():
        cls = getattr(lib, pyname)
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for field, _ in cls._fields_:
            lines.append(f'  printf("{cname} {field} %zu\\n", offsetof({cname}, {field}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    r = subprocess.run([cc, "-std=c11", "-I", str(ROOT / "include"), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr  # a ctypes field the header lacks fails here
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {}
    for ln in out:
        if ln:
            name, field, value = ln.split()
            got[(name, field)] = int(value)
    for cname, pyname in STRUCTS.items():
        cls = getattr(lib, pyname)
        assert got[(cname, "size")] == __import__("ctypes").sizeof(cls), cname
        for field, _ in cls._fields_:
            assert got[(cname, field)] == getattr(cls, field).offset, (cname, field)
