"""2D travel-time likelihood for many chains (C ABI mct_tt2d_*).

Mirrors the 2D code's likelihood call for travel times (datatype 0) and
travel plus differential times (datatype 1):
mcmc2d/likelihood_joint.f90:56 -> body_likelihood
(mcmc2d/likelihood_dd.F90:349-529), with the kdtree_to_grid call before it
(mcmc2d/mcmc.f90:1469-1525), and body_noise_likelihood
(mcmc2d/likelihood_dd.F90:32-106).
"""
import ctypes

import numpy as np

from ._lib import check, lib, ptr
from .surface import Grid


class TT2DSettings(ctypes.Structure):
    """fm2d settings (gridx, gridy, sgref, sgdic, sgext, order), sigdep,
    datatype, straight (isStraight) and the fm2d precision (0: FP64 in
    the reference's order, 1: double-float)."""
    _fields_ = [("gridx", ctypes.c_int), ("gridy", ctypes.c_int), ("sgref", ctypes.c_int), ("sgdic", ctypes.c_int),
                ("sgext", ctypes.c_int), ("order", ctypes.c_int), ("sigdep", ctypes.c_int),
                ("datatype", ctypes.c_int), ("straight", ctypes.c_int), ("precision", ctypes.c_int)]


class TT2DData(ctypes.Structure):
    _fields_ = [("nsrc", ctypes.c_int), ("nrev", ctypes.c_int), ("src", ctypes.c_void_p), ("rev", ctypes.c_void_p),
                ("raystat", ctypes.c_void_p), ("ttime", ctypes.c_void_p), ("sigma", ctypes.c_void_p),
                ("nrays", ctypes.c_int), ("dtime", ctypes.c_void_p), ("dcc", ctypes.c_void_p),
                ("ndtime", ctypes.c_int)]


class TravelTime2DLikelihood:
    """grid: dict as for SurfaceLikelihood (nz ignored); settings: the
    TT2DSettings fields; data: src (nsrc, 2), rev (nrev, 2), raystat and
    ttime (nsrc*nrev, source-major), optional sigma, nrays, and for
    datatype 1 dtime and dcc (ndd, nrev) with ndd = nsrc*(nsrc-1)/2 source
    pairs i<j in order, and ndtime."""

    def __init__(self, grid, settings, data, nslots, ncell_max):
        g = Grid(**grid)
        s = TT2DSettings(**settings)
        self.nsrc = int(data["nsrc"]) if "nsrc" in data else len(data["src"])
        src = np.ascontiguousarray(data["src"], np.float64).reshape(-1, 2)
        rev = np.ascontiguousarray(data["rev"], np.float64).reshape(-1, 2)
        rays = np.ascontiguousarray(data["raystat"], np.int32).ravel()
        tt = np.ascontiguousarray(data["ttime"], np.float64).ravel()
        sig = data.get("sigma")
        sig = None if sig is None else np.ascontiguousarray(sig, np.float64).ravel()
        dt = data.get("dtime")
        dt = None if dt is None else np.ascontiguousarray(dt, np.float64)
        dcc = data.get("dcc")
        dcc = None if dcc is None else np.ascontiguousarray(dcc, np.float64)
        self._keep = (src, rev, rays, tt, sig, dt, dcc)
        self.nrev = rev.shape[0]
        self.nsrc = src.shape[0]
        d = TT2DData(self.nsrc, self.nrev, src.ctypes.data, rev.ctypes.data, rays.ctypes.data, tt.ctypes.data,
                     None if sig is None else sig.ctypes.data, int(data.get("nrays", int((rays == 1).sum()))),
                     None if dt is None else dt.ctypes.data, None if dcc is None else dcc.ctypes.data,
                     int(data.get("ndtime", 0)))
        self.ncell_max = ncell_max
        h = ctypes.c_void_p()
        check("mct_tt2d_create", lib().mct_tt2d_create(ctypes.byref(g), ctypes.byref(s), ctypes.byref(d),
                                                       nslots, ncell_max, ctypes.byref(h)))
        self.h = h

    def set_priority(self, high):
        """Run this context's work on a high-priority (True) or a normal
        stream of the device."""
        check("mct_tt2d_set_priority", lib().mct_tt2d_set_priority(self.h, 1 if high else 0))

    def set_sm_share(self, share):
        """Keep this context's 2D travel-time kernels to a share (0-1) of the
        device's SMs (0 or 1: all of them); results do not depend on it."""
        check("mct_tt2d_set_sm_share", lib().mct_tt2d_set_sm_share(self.h, float(share)))

    def close(self):
        if self.h:
            lib().mct_tt2d_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def forward(self, ncells, points, params, n0, n1):
        """ncells (nch,), points (nch, ncell_max, 2), params (nch,
        ncell_max, 3), n0/n1 (nch, 2); returns (nch, 4): like, misfit,
        unweighted misfit, status."""
        ncells = np.ascontiguousarray(ncells, np.int32)
        nch = ncells.size
        points = np.ascontiguousarray(points, np.float64)
        params = np.ascontiguousarray(params, np.float64)
        n0 = np.ascontiguousarray(n0, np.float64).reshape(nch, 2)
        n1 = np.ascontiguousarray(n1, np.float64).reshape(nch, 2)
        out = np.zeros((nch, 4))
        check("mct_tt2d_forward", lib().mct_tt2d_forward(self.h, nch, ptr(ncells), ptr(points), ptr(params),
                                                         ptr(n0), ptr(n1), ptr(out)))
        return out

    def submit(self, ncells, points, params, n0, n1):
        """Starts forward() without waiting; poll() collects it."""
        ncells = np.ascontiguousarray(ncells, np.int32)
        nch = ncells.size
        points = np.ascontiguousarray(points, np.float64)
        params = np.ascontiguousarray(params, np.float64)
        n0 = np.ascontiguousarray(n0, np.float64).reshape(nch, 2)
        n1 = np.ascontiguousarray(n1, np.float64).reshape(nch, 2)
        check("mct_tt2d_submit", lib().mct_tt2d_submit(self.h, nch, ptr(ncells), ptr(points), ptr(params),
                                                       ptr(n0), ptr(n1)))
        self._pending = nch

    def poll(self):
        """(done, out): out (nchains, 4) once the submitted batch finished."""
        out = np.zeros((self._pending, 4))
        done = ctypes.c_int()
        check("mct_tt2d_poll", lib().mct_tt2d_poll(self.h, ptr(out), ctypes.byref(done)))
        return bool(done.value), (out if done.value else None)

    def commit(self, accept):
        """Chains with accept[c] keep the last forward as their state."""
        accept = np.ascontiguousarray(accept, np.int32)
        check("mct_tt2d_commit", lib().mct_tt2d_commit(self.h, accept.size, ptr(accept)))

    def noise_likelihood(self, n0, n1):
        """body_noise_likelihood of the 2D code on chains 0..nch-1's
        committed times with new n0/n1 (nch, 2)."""
        n0 = np.ascontiguousarray(n0, np.float64)
        nch = n0.shape[0]
        n0 = n0.reshape(nch, 2)
        n1 = np.ascontiguousarray(n1, np.float64).reshape(nch, 2)
        out = np.zeros((nch, 4))
        check("mct_tt2d_noise_likelihood", lib().mct_tt2d_noise_likelihood(self.h, nch, ptr(n0), ptr(n1), ptr(out)))
        return out

    def phase_time(self, index):
        """Last forward's times (nsrc, nrev) of batch position index."""
        out = np.zeros((self.nsrc, self.nrev))
        check("mct_tt2d_phase_time", lib().mct_tt2d_phase_time(self.h, int(index), ptr(out)))
        return out
