"""The C-ABI library loads without a GPU and exports every function that the
headers under include/ declare (CPU only: no compute calls)."""
import ctypes
import glob
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = sorted(glob.glob(os.path.join(ROOT, "include", "**", "*.h"), recursive=True))


def declared_functions():
    names = set()
    for h in HEADERS:
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        src = re.sub(r"//[^\n]*", "", src)
        src = re.sub(r"#ifdef __cplusplus.*?#endif", "", src, flags=re.S)
        src = re.sub(r"#[^\n]*", "", src)
        # drop struct / enum bodies
        while True:
            n = re.sub(r"\{[^{}]*\}", ";", src)
            if n == src:
                break
            src = n
        for stmt in src.split(";"):
            s = " ".join(stmt.split())
            if not s or s.startswith("typedef") or "(" not in s:
                continue
            m = re.match(r"^(?:extern\s+)?[\w\s\*]+?\b(\w+)\s*\(", s)
            if m and m.group(1) not in ("if", "while", "sizeof"):
                names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def libpath():
    import __graft_entry__ as g
    from quantum_geometric_tensor_gb300 import LIB_PATH
    if not os.path.exists(LIB_PATH):
        g.build()
    return LIB_PATH


def test_headers_parsed():
    names = declared_functions()
    for must in ("qgt_plan_create", "geometric_compute_full_qgt", "compute_quantum_geometric_tensor",
                 "geometric_compute_fubini_study_metric", "compute_regularized_natural_gradient",
                 "geometric_tensor_create", "diffgeo_compute_fubini_study", "compute_natural_gradient_gpu"):
        assert must in names


def test_library_loads_and_exports_every_declared_symbol(libpath):
    lib = ctypes.CDLL(libpath)
    out = subprocess.run(["nm", "-D", "--defined-only", libpath], capture_output=True, text=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if ln.strip()}
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, f"declared but not exported: {missing}"
    for n in declared_functions():
        getattr(lib, n)


def test_no_oracle_linkage(libpath):
    out = subprocess.run(["nm", "-D", libpath], capture_output=True, text=True).stdout
    assert "or_derivatives" not in out and "ref_simulate" not in out
    ldd = subprocess.run(["ldd", libpath], capture_output=True, text=True).stdout
    assert "oracle" not in ldd


def test_version_string(libpath):
    lib = ctypes.CDLL(libpath)
    lib.qgt_version.restype = ctypes.c_char_p
    assert b"sm_103a" in lib.qgt_version()
