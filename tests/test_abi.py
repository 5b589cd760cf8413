"""The C ABI library loads and exports every symbol include/pfg.h declares
(no compute calls: this runs without a GPU)."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "pfg.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"\b(pfg_[a-z0-9_]+)\s*\(", src)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    from plantfem_gb300 import _native
    if not os.path.exists(_native.LIB_PATH):
        from plantfem_gb300.build import build
        build()
    return ctypes.CDLL(_native.LIB_PATH)


def test_header_declares_functions():
    names = declared_functions()
    assert "pfg_solve" in names and "pfg_crs_spmv_real64" in names and len(names) >= 20


def test_every_declared_symbol_is_exported(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"declared in pfg.h but not exported: {missing}"


def test_python_binding_covers_header():
    from plantfem_gb300 import _native
    missing = [n for n in declared_functions() if n not in _native.SIGNATURES]
    assert not missing, f"no ctypes signature for: {missing}"


def test_exports_are_c_linkage(lib):
    from plantfem_gb300 import _native
    out = subprocess.run(["nm", "-D", "--defined-only", _native.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (pfg_[a-z0-9_]+)\b", out))
    assert set(declared_functions()) <= exported


def test_version_and_defaults_without_gpu(lib):
    from plantfem_gb300 import _native
    L = _native.load()
    assert b"sm_103a" in L.pfg_version()
    o = _native.default_opts()
    # the reference's FEMSolver_ defaults (FEMSolverClass.f90:69-71)
    assert o.itrmax == 100000 and o.er0 == 1e-10 and o.relative_er == 1e-10
    assert o.algorithm == _native.ALG_BICGSTAB and o.precision == _native.PREC_FP64
