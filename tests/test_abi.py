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


def _header_struct_fields(name):
    """(type, field) pairs of `typedef struct <name> {...}` in include/pfg.h, in order."""
    import re
    txt = open(HEADER).read()
    body = re.search(r"typedef struct %s \{(.*?)\} %s;" % (name, name), txt, re.S).group(1)
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    out = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        parts = decl.split()
        ctype, names = parts[0], " ".join(parts[1:])
        for nm in names.split(","):
            out.append((ctype, nm.strip()))
    return out


@pytest.mark.parametrize("cname,pyname", [("pfg_solve_opts", "SolveOpts"), ("pfg_info", "Info"),
                                          ("pfg_eig_opts", "EigOpts"), ("pfg_newmark_params", "NewmarkParams"),
                                          ("pfg_batch_config", "BatchConfig"), ("pfg_batch_info", "BatchInfo")])
def test_ctypes_structs_match_header(cname, pyname):
    """Every struct the Python layer passes by pointer has the header's fields in
    the header's order, with matching C types."""
    import ctypes as C
    from plantfem_gb300 import _native as N
    sizes = {"int32_t": C.c_int32, "int64_t": C.c_int64, "uint64_t": C.c_uint64, "double": C.c_double}
    hdr = _header_struct_fields(cname)
    fields = getattr(N, pyname)._fields_
    assert len(hdr) == len(fields), (cname, hdr, fields)
    for (ctype, name), (pyfield, pytype) in zip(hdr, fields):
        assert name.lower() == pyfield.lower() or name.replace("_", "").lower() == pyfield.replace("_", "").lower(), \
            (cname, name, pyfield)
        if ctype in sizes:
            assert C.sizeof(pytype) == C.sizeof(sizes[ctype]), (cname, name)


# ------------------------------------------------- the Fortran binding module
F90 = os.path.join(ROOT, "include", "FEMSolverGPUClass.f90")
_F2C = {"c_int32_t": ("int32_t",), "c_int": ("int32_t", "int"), "c_double": ("double",),
        "c_int64_t": ("int64_t", "uint64_t"), "c_size_t": ("size_t",)}


def _f90_source():
    return re.sub(r"!.*", "", open(F90).read())  # drop comments


def _f90_bindc_types():
    """{name: [(kind, field), ...]} of the `type, bind(C) :: name` blocks, in order."""
    out = {}
    for name, body in re.findall(r"type\s*,\s*bind\(C\)\s*::\s*(\w+)(.*?)end\s+type", _f90_source(), re.S | re.I):
        fields = []
        for line in body.strip().splitlines():
            m = re.match(r"\s*(?:integer|real)\((\w+)\)\s*::\s*(.*)", line)
            if m:
                fields += [(m.group(1), f.strip()) for f in m.group(2).split(",")]
        out[name] = fields
    return out


@pytest.mark.parametrize("cname", ["pfg_solve_opts", "pfg_info", "pfg_eig_opts"])
def test_fortran_bindc_types_match_header(cname):
    """The Fortran module's bind(C) types have the header's fields, in order,
    with interoperable kinds of the same size."""
    hdr = _header_struct_fields(cname)
    f90 = _f90_bindc_types()[cname]
    assert len(hdr) == len(f90), (cname, hdr, f90)
    for (ctype, name), (kind, fname) in zip(hdr, f90):
        assert name.lower() == fname.lower(), (cname, name, fname)
        assert ctype in _F2C[kind], (cname, name, ctype, kind)


def _c_prototype_arity():
    src = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    out = {}
    for name, args in re.findall(r"\b(pfg_[a-z0-9_]+)\s*\(([^)]*)\)\s*;", src):
        a = args.strip()
        out[name] = 0 if a in ("", "void") else a.count(",") + 1
    return out


def test_fortran_interfaces_bind_declared_symbols():
    """Every bind(C, name=...) of the Fortran module names a function that
    include/pfg.h declares, with as many dummy arguments as the C prototype."""
    src = _f90_source()
    ar = _c_prototype_arity()
    found = re.findall(r"(?:function|subroutine)\s+(\w+)\s*\(([^)]*)\)\s*(?:&\s*)?bind\(C\s*,\s*name\s*=\s*\"(\w+)\"\)",
                       src, re.I)
    assert len(found) >= 25
    for fname, dummies, cname in found:
        assert fname == cname
        assert cname in ar, cname
        n = 0 if not dummies.strip() else dummies.count(",") + 1
        assert n == ar[cname], (cname, n, ar[cname])


def test_fortran_type_bound_names_mirror_femsolver():
    """FEMSolverGPU_ offers the FEMSolver_ procedures the GPU path covers."""
    src = _f90_source()
    bound = set(re.findall(r"procedure\s*,\s*public\s*::\s*(\w+)\s*=>", src, re.I))
    assert {"init", "setDomain", "setCRS", "setRHS", "setMatrix", "setVector", "fix", "solve", "zeros",
            "keepThisMatrixAs", "loadMatrix", "fix_eig", "eig", "getCRS", "remove"} <= bound
