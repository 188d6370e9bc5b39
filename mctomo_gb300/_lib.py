"""ctypes binding of libmctomo_gpu.so (the C ABI in include/mctomo.h).

The library is built in-tree by ``mctomo_gb300.build``. There is no CPU
fallback: if the shared library is missing or fails to load, every call
raises ``MctError``.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmctomo_gpu.so")

MCT_OK = 0
MCT_MODEL_INVALID = 1
ERRORS = {
    -1: "MCT_ERR_ARG", -2: "MCT_ERR_CUDA", -3: "MCT_ERR_NOMEM", -4: "MCT_ERR_OUTSIDE",
    -5: "MCT_ERR_UNSUPPORTED", -6: "MCT_ERR_TIMEOUT", -7: "MCT_ERR_INTERNAL",
}

P = ctypes.c_void_p
I = ctypes.c_int
D = ctypes.c_double
ULLP = ctypes.POINTER(ctypes.c_ulonglong)

class ModesPara(ctypes.Structure):
    """mct_modes_para: the reference's T_MODES_PARA (surfmodes/surfmodes.f90:23-30)."""
    _fields_ = [("modetype", ctypes.c_int), ("nmodes", ctypes.c_int), ("phase_group", ctypes.c_int),
                ("tolmin", ctypes.c_double), ("tolmax", ctypes.c_double), ("smin_min", ctypes.c_double),
                ("smin_max", ctypes.c_double), ("dc", ctypes.c_double), ("dcm", ctypes.c_double),
                ("dc1", ctypes.c_double), ("dc2", ctypes.c_double)]


# name -> (restype, argtypes); must list every symbol declared in include/mctomo.h
SIGNATURES = {
    "mct_version": (ctypes.c_char_p, []),
    "mct_last_error": (ctypes.c_char_p, []),
    "mct_kdtree_to_grid": (I, [I, I, P, P, I, I, I, P, P, P, P, P, P, P]),
    "mct_grid_nearest_batch_device": (I, [I, I, I, P, P, P, I, I, I, P, P, P, P, P, P, P, P]),
    "mct_grid_nearest_batch_device_noalloc": (I, [I, I, I, P, P, P, I, I, I, P, P, P, P, P, P, P, P]),
    "mct_grid_status": (I, [P, P]),
    "mct_surfdisp96": (I, [P, P, P, P, I, I, I, I, I, I, P, D, P, P, P]),
    "mct_surfdisp_mmodes": (I, [P, P, P, P, I, I, I, I, I, I, P, D, P, P, P]),
    "mct_surfmodes": (I, [P, P, P, P, I, P, I, I, I, D, P, P, P]),
    "mct_surfmodes_para": (I, [P, P, P, P, I, P, I, P, P, P, P]),
    "mct_grt_batch": (I, [I, I, P, P, P, P, P, I, P, P, P, P, P, ULLP]),
    "mct_surfmodes_route": (I, [I, I, P, P, P, I, P]),
    "mct_grt_batch_device": (I, [I, I, P, P, P, P, P, I, P, P, P, P, P, P, P]),
    "mct_surfdisp_batch": (I, [I, I, P, P, P, P, P, I, P, I, I, I, D, I, I, P, P, P, P]),
    "mct_surfdisp_batch_device": (I, [I, I, P, P, P, P, P, I, P, I, I, I, D, I, I, P, P, P, P, P]),
    "mct_modrays": (I, [I, P, P, I, P, P, P, I, I, I, D, D, D, D, P, I, I, I, I, I, D, I, D, P, I, P, P]),
    "mct_modrays_batch": (I, [I, I, P, P, I, P, P, I, P, I, I, D, D, D, D, P, I, I, I, I, I, I, P, P, I]),
    "mct_modrays_group_batch": (I, [I, I, P, P, I, P, P, I, P, I, I, D, D, D, D, P, P, I, I, I, I, I, I, P, P, P, P,
                                    I]),
    "mct_fast_marching3d": (I, [I, I, I, D, D, D, D, D, D, P, P, P, I, I, P, P]),
    "mct_eikonal3d_batch": (I, [I, I, I, I, D, D, D, D, D, D, I, P, P, P, I, P, I, P, P, P]),
    "mct_eik3_tile_config": (I, [I, I, I, I, I]),
    "mct_body_create": (I, [P, P, P, I, I, P]),
    "mct_body_destroy": (I, [P]),
    "mct_body_forward": (I, [P, I, P, P, P, P, P, P, P]),
    "mct_body_phase_time": (I, [P, I, P, P]),
    "mct_body_submit": (I, [P, I, P, P, P, P, P, P]),
    "mct_body_location_likelihood": (I, [P, I, P, P, P, P, P]),
    "mct_body_location_commit": (I, [P, I, P]),
    "mct_body_poll": (I, [P, P, P]),
    "mct_body_commit": (I, [P, I, P]),
    "mct_body_noise_likelihood": (I, [P, I, P, P, P, P]),
    "mct_tt2d_create": (I, [P, P, P, I, I, P]),
    "mct_tt2d_destroy": (I, [P]),
    "mct_tt2d_forward": (I, [P, I, P, P, P, P, P, P]),
    "mct_tt2d_commit": (I, [P, I, P]),
    "mct_tt2d_noise_likelihood": (I, [P, I, P, P, P]),
    "mct_tt2d_phase_time": (I, [P, I, P]),
    "mct_tt2d_submit": (I, [P, I, P, P, P, P, P]),
    "mct_tt2d_poll": (I, [P, P, P]),
    "mct_surf_set_priority": (I, [P, I]),
    "mct_body_set_priority": (I, [P, I]),
    "mct_tt2d_set_priority": (I, [P, I]),
    "mct_surf_set_sm_share": (I, [P, D]),
    "mct_tt2d_set_sm_share": (I, [P, D]),
    "mct_rng_create": (I, [ctypes.c_uint, P]),
    "mct_rng_destroy": (None, [P]),
    "mct_rng_seed": (I, [P, ctypes.c_uint]),
    "mct_rng_unirand": (D, [P]),
    "mct_rng_gasdev": (D, [P]),
    "mct_rng_u32": (ctypes.c_uint, [P]),
    "mct_rng_count": (ctypes.c_longlong, [P]),
    "mct_mcmc_propose": (I, [P, P, I, I, P, P]),
    "mct_mcmc_accept": (I, [P, P, D, D]),
    "mct_mcmc_accept_tempered": (I, [P, P, D, D, D]),
    "mct_pt_init": (I, [P]),
    "mct_mcmc_record": (I, [P, P, I, D, D, D, P]),
    "mct_samples_write": (I, [ctypes.c_char_p, I, P, I]),
    "mct_samples_read": (I, [ctypes.c_char_p, I, P, I]),
    "mct_pt_choose": (I, [P, P, P, P]),
    "mct_pt_swap": (I, [P, P, I, I, D, D]),
    "mct_surf_create": (I, [P, P, P, I, I, P]),
    "mct_surf_destroy": (I, [P]),
    "mct_surf_forward": (I, [P, I, P, P, P, P, P, P, P]),
    "mct_surf_commit": (I, [P, P]),
    "mct_surf_forward_device": (I, [P, I, P, P, P, P, P, P, P, P]),
    "mct_surf_commit_device": (I, [P, P, P]),
    "mct_surf_phase_time": (I, [P, I, P, P]),
    "mct_surf_noise_likelihood": (I, [P, I, P, P, P, P]),
    "mct_surf_stream": (I, [P, P]),
    "mct_surf_device_bytes": (I, [P, P, P, I, I, P]),
    "mct_surf_admit": (I, [P, P]),
    "mct_surf_evict": (I, [P, I]),
    "mct_surf_submit": (I, [P, I, P, P, P, P, P, P]),
    "mct_surf_poll": (I, [P, P, P]),
    "mct_surf_stat_add": (I, [P, I, P]),
    "mct_surf_stat_read": (I, [P, I, P, P, P, P, P]),
    "mct_surf_stat_reset": (I, [P, I]),
    "mct_surf_profile_start": (I, [P, I]),
    "mct_surf_profile_read": (I, [P, P, P, P]),
}


class MctError(RuntimeError):
    """A negative status from the library (or the library is unavailable)."""

    def __init__(self, name, code, msg=""):
        self.code = code
        super().__init__("%s failed: %s (%s) %s" % (name, code, ERRORS.get(code, "?"), msg))


_lib = None


def lib():
    """Load (once) and return the bound library."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise MctError("load", -2, "libmctomo_gpu.so not built at %s; run mctomo_gb300.build.build()" % LIB_PATH)
    try:
        handle = ctypes.CDLL(LIB_PATH)
    except OSError as e:  # pragma: no cover - depends on the host
        raise MctError("load", -2, str(e))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(handle, name)
        fn.restype = res
        fn.argtypes = args
    _lib = handle
    return _lib


def check(name, rc):
    """Raise on a negative status; return the status otherwise (0 or 1)."""
    if rc < 0:
        msg = lib().mct_last_error().decode(errors="replace")
        raise MctError(name, rc, msg)
    return rc


def ptr(a):
    """Pointer to a numpy array's data (None passes NULL)."""
    if a is None:
        return None
    return ctypes.c_void_p(a.ctypes.data)
