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
    for m in re.finditer(r"\b(?:int|void|double|unsigned|long long|const char \*)\s*\**\s*(mct_\w+)\s*\(([^)]*)\)\s*;",
                         h):
        funcs[m.group(1)] = [a.strip() for a in m.group(2).split(",") if a.strip() and a.strip() != "void"]
    structs = {}
    for m in re.finditer(r"typedef struct\s*\{(.*?)\}\s*(\w+)\s*;", h, flags=re.S):
        fields = []
        for decl in m.group(1).split(";"):
            decl = decl.strip()
            if not decl:
                continue
            if decl.startswith("long long"):
                kind, names = "long long", decl[len("long long"):]
            else:
                kind = "ptr" if "*" in decl else decl.split()[0]
                names = decl.replace("*", " ").split(None, 1 if not decl.startswith("const") else 2)[-1]
            fields += [(kind, n.strip().replace("[", "(").replace("]", ")")) for n in names.split(",")]
        structs[m.group(2)] = fields
    return funcs, structs


def test_fortran_module_covers_the_header():
    # include/mctomo.f90: one bind(C) interface per C entry point, with the
    # C parameter count, and bind(C) types laid out as the C structs
    import re
    funcs, structs = _c_decls()
    f = open(os.path.join(ROOT, "include", "mctomo.f90")).read()
    ff = {}
    for m in re.finditer(r'(?:function|subroutine)\s+(mct_\w+)\s*\(([^)]*)\)\s*(?:&\s*)?bind\(C,\s*name="(\w+)"\)',
                         f, flags=re.S):
        assert m.group(1) == m.group(3)
        ff[m.group(1)] = [a for a in m.group(2).replace("&", "").split(",") if a.strip()]
    assert set(ff) == set(funcs)
    for name, args in funcs.items():
        assert len(ff[name]) == len(args), name
    kinds = {"integer(c_int)": "int", "real(c_double)": "double", "type(c_ptr)": "ptr",
             "integer(c_long_long)": "long long"}
    for m in re.finditer(r"type, bind\(C\) :: (\w+)\n(.*?)end type", f, flags=re.S):
        fields = []
        for line in m.group(2).strip().splitlines():
            t, names = line.split("::")
            fields += [(kinds[t.strip()], n.strip()) for n in names.split(",")]
        assert fields == structs[m.group(1)], m.group(1)
    assert set(structs) == set(re.findall(r"type, bind\(C\) :: (\w+)", f))


def test_null_contexts_and_bad_sizes_are_refused_without_a_gpu(gpulib):
    # every context call checks its handle and sizes before touching the
    # device, so these return MCT_ERR_ARG (-1) on a machine without a GPU
    import numpy as np
    L = gpulib
    N = None
    d = np.zeros(16)
    i = np.zeros(16, np.int32)
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    calls = {
        "mct_surf_forward": lambda: L.mct_surf_forward(N, 1, P(i), P(i), P(d), P(d), P(d), P(d), P(d)),
        "mct_surf_commit": lambda: L.mct_surf_commit(N, P(i)),
        "mct_surf_forward_device": lambda: L.mct_surf_forward_device(N, 1, N, N, N, N, N, N, N, N),
        "mct_surf_commit_device": lambda: L.mct_surf_commit_device(N, N, N),
        "mct_surf_noise_likelihood": lambda: L.mct_surf_noise_likelihood(N, 1, P(i), P(d), P(d), P(d)),
        "mct_surf_phase_time": lambda: L.mct_surf_phase_time(N, 0, P(d), P(d)),
        "mct_surf_profile_start": lambda: L.mct_surf_profile_start(N, 1),
        "mct_surf_profile_read": lambda: L.mct_surf_profile_read(N, P(d), P(i), P(d)),
        "mct_surf_stream": lambda: L.mct_surf_stream(N, P(d)),
        "mct_surf_admit": lambda: L.mct_surf_admit(N, P(i)),
        "mct_surf_evict": lambda: L.mct_surf_evict(N, 0),
        "mct_surf_submit": lambda: L.mct_surf_submit(N, 1, P(i), P(i), P(d), P(d), P(d), P(d)),
        "mct_surf_poll": lambda: L.mct_surf_poll(N, P(d), P(i)),
        "mct_surf_create": lambda: L.mct_surf_create(N, N, N, 1, 1, N),
        "mct_surf_device_bytes": lambda: L.mct_surf_device_bytes(N, N, N, 1, 1, N),
        "mct_body_create": lambda: L.mct_body_create(N, N, N, 1, 1, N),
        "mct_body_forward": lambda: L.mct_body_forward(N, 1, P(i), P(d), P(d), P(d), P(d), P(d), P(d)),
        "mct_body_commit": lambda: L.mct_body_commit(N, 1, P(i)),
        "mct_body_noise_likelihood": lambda: L.mct_body_noise_likelihood(N, 1, P(d), P(d), P(d), P(d)),
        "mct_body_phase_time": lambda: L.mct_body_phase_time(N, 0, P(d), P(i)),
        "mct_tt2d_forward": lambda: L.mct_tt2d_forward(N, 1, P(i), P(d), P(d), P(d), P(d), P(d)),
        "mct_tt2d_commit": lambda: L.mct_tt2d_commit(N, 1, P(i)),
        "mct_tt2d_noise_likelihood": lambda: L.mct_tt2d_noise_likelihood(N, 1, P(d), P(d), P(d)),
        "mct_tt2d_phase_time": lambda: L.mct_tt2d_phase_time(N, 0, P(d)),
        "mct_kdtree_to_grid": lambda: L.mct_kdtree_to_grid(4, 1, P(d), P(d), 2, 2, 2, P(d), P(d), N, P(i), P(d), P(d),
                                                           P(d)),
        "mct_surfdisp_batch": lambda: L.mct_surfdisp_batch(1, 1, P(i), P(d), P(d), P(d), P(d), 61, P(d), 2, 1, 0,
                                                           0.001, 0, 0, P(d), P(d), P(i), N),
        "mct_surfmodes": lambda: L.mct_surfmodes(P(d), P(d), P(d), P(d), 0, P(d), 1, 0, 0, 0.001, P(d), P(d), P(i)),
        "mct_eikonal3d_batch": lambda: L.mct_eikonal3d_batch(0, 2, 2, 2, 1., 1., 1., 0., 0., 0., 1, P(d), P(i),
                                                             P(d), 0, P(d), 0, P(d), N, P(i)),
    }
    for name, call in calls.items():
        assert call() == -1, name
    # destroying a null context is a no-op
    assert L.mct_surf_destroy(N) == 0 and L.mct_body_destroy(N) == 0 and L.mct_tt2d_destroy(N) == 0


def test_header_is_strict_c99_and_cxx(tmp_path):
    # the C ABI header compiles as ISO C99 and C++11 with warnings as errors,
    # and a C program can take every declared entry point's address
    import shutil
    import subprocess
    if not shutil.which("gcc") or not shutil.which("g++"):
        import pytest
        pytest.skip("no host C compiler")
    syms = declared_symbols()
    src = tmp_path / "abi.c"
    body = "\n".join("  p[%d] = (void (*)(void))%s;" % (i, s) for i, s in enumerate(syms))
    src.write_text('#include "mctomo.h"\nint main(void) {\n  void (*p[%d])(void);\n%s\n  return p[0] == 0;\n}\n'
                   % (len(syms), body))
    inc = "-I" + os.path.join(ROOT, "include")
    for cmd in (["gcc", "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", inc, "-c", str(src), "-o",
                 str(tmp_path / "a.o")],
                ["g++", "-std=c++11", "-Wall", "-Wextra", "-pedantic", "-Werror", inc, "-x", "c++", "-c", str(src),
                 "-o", str(tmp_path / "b.o")]):
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
