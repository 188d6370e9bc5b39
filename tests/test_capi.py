"""CPU tests of the C ABI library: it builds, loads without a GPU, and exports
every entry point include/mctomo.h declares."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "mctomo.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(mct_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol(gpulib):
    from mctomo_gb300 import _lib
    handle = ctypes.CDLL(_lib.LIB_PATH)
    syms = declared_symbols()
    assert len(syms) >= 8
    for s in syms:
        assert hasattr(handle, s), s
    # the Python binding lists exactly the declared symbols
    assert sorted(_lib.SIGNATURES) == syms


def test_version_and_error_calls_work_without_gpu(gpulib):
    assert b"sm_103a" in gpulib.mct_version()
    assert isinstance(gpulib.mct_last_error(), bytes)


def test_argument_errors_are_reported_not_fatal(gpulib):
    import numpy as np
    from mctomo_gb300 import MctError, surfdisp96
    try:
        surfdisp96(np.ones(2), np.ones(2), np.ones(2), np.ones(2), iwave=2, igr=0, t=np.ones(3),
                   dphase=0.0)
    except MctError as e:
        assert e.code == -1
    else:
        raise AssertionError("expected MctError")


def _c_decls():
    import re
    h = open(os.path.join(ROOT, "include", "mctomo.h")).read()
    h = re.sub(r"/\*.*?\*/", "", h, flags=re.S)
    funcs = {}
    for m in re.finditer(r"\b(?:int|const char \*)\s*\**\s*(mct_\w+)\s*\(([^)]*)\)\s*;", h):
        funcs[m.group(1)] = [a.strip() for a in m.group(2).split(",") if a.strip() and a.strip() != "void"]
    structs = {}
    for m in re.finditer(r"typedef struct\s*\{(.*?)\}\s*(\w+)\s*;", h, flags=re.S):
        fields = []
        for decl in m.group(1).split(";"):
            decl = decl.strip()
            if not decl:
                continue
            kind = "ptr" if "*" in decl else decl.split()[0]
            names = decl.replace("*", " ").split(None, 1 if not decl.startswith("const") else 2)[-1]
            fields += [(kind, n.strip()) for n in names.split(",")]
        structs[m.group(2)] = fields
    return funcs, structs


def test_fortran_module_covers_the_header():
    # include/mctomo.f90: one bind(C) interface per C entry point, with the
    # C parameter count, and bind(C) types laid out as the C structs
    import re
    funcs, structs = _c_decls()
    f = open(os.path.join(ROOT, "include", "mctomo.f90")).read()
    ff = {}
    for m in re.finditer(r'function\s+(mct_\w+)\s*\(([^)]*)\)\s*(?:&\s*)?bind\(C,\s*name="(\w+)"\)', f, flags=re.S):
        assert m.group(1) == m.group(3)
        ff[m.group(1)] = [a for a in m.group(2).replace("&", "").split(",") if a.strip()]
    assert set(ff) == set(funcs)
    for name, args in funcs.items():
        assert len(ff[name]) == len(args), name
    kinds = {"integer(c_int)": "int", "real(c_double)": "double", "type(c_ptr)": "ptr"}
    for m in re.finditer(r"type, bind\(C\) :: (\w+)\n(.*?)end type", f, flags=re.S):
        fields = []
        for line in m.group(2).strip().splitlines():
            t, names = line.split("::")
            fields += [(kinds[t.strip()], n.strip()) for n in names.split(",")]
        assert fields == structs[m.group(1)], m.group(1)
    assert set(structs) == set(re.findall(r"type, bind\(C\) :: (\w+)", f))
