"""Build and load the oracle shared libraries (test infrastructure only)."""
import ctypes
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SOURCES = ["kdgrid.cpp", "surfdisp.cpp", "fm2d.cpp", "sfmm3d.cpp", "likelihood.cpp", "surf_pipeline.cpp",
           "grt.cpp"]
LIB = os.path.join(HERE, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libfmm_ref.so")

_P = ctypes.c_void_p
_I = ctypes.c_int
_D = ctypes.c_double
_F = ctypes.c_float
_LL = ctypes.c_longlong


def build(force=False):
    """Compile liboracle.so from the restatements in this directory."""
    srcs = [os.path.join(HERE, s) for s in SOURCES]
    if not force and os.path.exists(LIB):
        mt = os.path.getmtime(LIB)
        if all(os.path.getmtime(s) <= mt for s in srcs + [os.path.join(HERE, "oracle.h")]):
            return LIB
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fopenmp",
           "-fPIC", "-shared", "-o", LIB] + srcs
    subprocess.check_call(cmd, cwd=HERE)
    return LIB


def build_reference():
    """Compile the reference's fastMarching3D from its own sources (only where
    the reference tree is present). Returns the path or None."""
    script = os.path.join(HERE, "build_ref.sh")
    # the recipe locates the reference tree itself (MCT_REFERENCE overrides)
    # and exits with status 2 where it is absent
    rc = subprocess.call(["bash", script], cwd=HERE)
    if rc == 2:
        return REF_LIB if os.path.exists(REF_LIB) else None
    if rc != 0:
        raise subprocess.CalledProcessError(rc, script)
    return REF_LIB


_lib = None


def load():
    global _lib
    if _lib is None:
        build()
        lib = ctypes.CDLL(LIB)
        sig = {
            "orc_kdtree_to_grid": (_I, [_I, _I, _P, _P, _I, _I, _I, _D, _D, _D, _D, _D, _D,
                                        _I, _I, _I, _I, _I, _I, _P, _P, _P, _P]),
            "orc_kdtree_nearest": (_I, [_I, _I, _P, _P]),
            "orc_surfdisp96": (_I, [_P, _P, _P, _P, _I, _I, _I, _I, _I, _P, _D, _P, _P, _P]),
            "orc_grt_modes": (_I, [_I, _P, _P, _P, _P, _I, _P, _I, _I, _D, _D, _D, _D, _D, _D, _D, _P, _P, _P]),
            "orc_grt_nlvls1": (_I, [_I, _P, _P, _P, _P, _I]),
            "orc_grt_secfun": (_D, [_I, _P, _P, _P, _P, _I, _D, _D, _P]),
            "orc_surfdisp_mmodes": (_I, [_P, _P, _P, _P, _I, _I, _I, _I, _I, _P, _D, _P, _P, _P]),
            "orc_dltar": (_D, [_D, _D, _I, _P, _P, _P, _P, _I]),
            "orc_gtsolh": (_F, [_F, _F]),
            "orc_count_lvl": (_I, [_P, _P, _I, _I]),
            "orc_surfmodes": (_I, [_P, _P, _P, _P, _I, _P, _I, _I, _I, _D, _P, _P, _P]),
            "orc_modrays": (_I, [_I, _P, _P, _I, _P, _P, _P, _I, _I, _D, _D, _D, _D, _P,
                                 _I, _I, _I, _I, _I, _I, _D, _P, _P]),
            "orc_modrays_group": (_I, [_I, _P, _P, _I, _P, _P, _P, _I, _I, _D, _D, _D, _D, _P,
                                       _I, _I, _I, _I, _I, _I, _P, _P, _P, _P, _P]),
            "orc_surf_likelihood_ex": (_I, [_P, _P, _P, _D, _D, _I, _P, _P, _I, _P, _I, _P, _I, _P, _P, _P, _P, _I,
                                            _P, _P, _P, _I, _I, _P, _P, _P, _P, _P]),
            "orc_straight_group": (_I, [_I, _P, _I, _P, _P, _I, _I, _D, _D, _D, _D, _P, _P, _P]),
            "orc_fm2d_trace": (_I, [_I, _P, _P, _I]),
            "orc_fm2d_trace_count": (_I, []),
            "orc_fast_marching3d": (_I, [_I, _I, _I, _D, _D, _D, _D, _D, _D, _P, _P, _P, _I,
                                         _I, _P, _P]),
            "orc_check_model": (_I, [_P, _I, _I, _I]),
            "orc_convert_to_layer": (_I, [_P, _P, _P, _I, _D, _D, _D, _P, _P, _P, _P]),
            "orc_surf_misfit": (_I, [_I, _I, _I, _P, _P, _P, _P, _I, _P, _P, _I, _P, _P]),
            "orc_body_misfit": (_I, [_I, _I, _I, _P, _P, _P, _P, _P, _I, _P, _P, _I, _P, _P]),
            "orc_location_times": (_I, [_I, _I, _I, _D, _D, _D, _D, _D, _D, _D, _I, _I, _I, _P, _P, _P]),
            "orc_tt2d_misfit": (_I, [_I, _I, _P, _P, _P, _P, _I, _I, _P, _P, _I, _P, _P, _I, _P]),
            "orc_tt2d_noise": (_I, [_I, _I, _P, _P, _P, _P, _I, _P, _P, _I, _P, _P, _I, _P]),
            "orc_surf_likelihood": (_I, [_P, _P, _P, _D, _D, _I, _P, _P, _I, _P, _I, _P, _I, _P,
                                         _P, _P, _P, _I, _P, _P, _P, _P, _P, _P]),
            "orc_vs2vp": (_D, [_D]),
            "orc_vp2rho": (_D, [_D]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def load_reference():
    """The reference's own fastMarching3D, or None where it was not built."""
    if not os.path.exists(REF_LIB):
        return None
    lib = ctypes.CDLL(REF_LIB)
    fn = lib.fastMarching3D
    fn.restype = _I
    fn.argtypes = [_I, _I, _I, _D, _D, _D, _D, _D, _D, _P, _P, _P, _I, _I, _P, _P]
    return lib
