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
