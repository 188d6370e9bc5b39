"""Body-wave (P, S) likelihood for many chains (C ABI mct_body_*).

Mirrors the reference's likelihood() for datatypes 0/1
(src/likelihood.f90:57-93 -> src/likelihood_body.F90:151-337).
"""
import ctypes

import numpy as np

from ._lib import check, lib, ptr
from .surface import Grid


class BodySettings(ctypes.Structure):
    """order, np, sigdep as the reference's settings; solver selects the 3D
    travel-time solver (0 default: the exact heap march for order 1, tiles
    for order 0; EIK3_TILES or EIK3_HEAP)."""
    _fields_ = [("order", ctypes.c_int), ("np", ctypes.c_int), ("sigdep", ctypes.c_int),
                ("solver", ctypes.c_int), ("dynamic", ctypes.c_int)]


class BodyData(ctypes.Structure):
    _fields_ = [("nsrc", ctypes.c_int), ("nrev", ctypes.c_int), ("np", ctypes.c_int),
                ("rev", ctypes.c_void_p), ("raystat", ctypes.c_void_p), ("ttime", ctypes.c_void_p),
                ("sigma", ctypes.c_void_p), ("nrays", ctypes.c_int)]


class BodyLikelihood:
    """grid: dict as for SurfaceLikelihood; settings: order, np, sigdep;
    data: nsrc, rev (nrev, 3), raystat (np, nsrc*nrev), ttime (np, nsrc*nrev),
    optional sigma."""

    def __init__(self, grid, settings, data, nslots, ncell_max):
        g = Grid(**grid)
        s = BodySettings(**settings)
        self.np = settings["np"]
        self.nsrc = int(data["nsrc"])
        rev = np.ascontiguousarray(data["rev"], np.float64)
        rays = np.ascontiguousarray(data["raystat"], np.int32)
        tt = np.ascontiguousarray(data["ttime"], np.float64)
        sig = data.get("sigma")
        sig = None if sig is None else np.ascontiguousarray(sig, np.float64)
        self._keep = (rev, rays, tt, sig)
        self.nrev = rev.shape[0]
        d = BodyData(self.nsrc, self.nrev, self.np, rev.ctypes.data, rays.ctypes.data, tt.ctypes.data,
                     None if sig is None else sig.ctypes.data, int(data.get("nrays", int((rays == 1).sum()))))
        self.ncell_max = ncell_max
        h = ctypes.c_void_p()
        check("mct_body_create", lib().mct_body_create(ctypes.byref(g), ctypes.byref(s), ctypes.byref(d),
                                                       nslots, ncell_max, ctypes.byref(h)))
        self.h = h

    def set_priority(self, high):
        """Run this context's work on a high-priority (True) or a normal
        stream of the device."""
        check("mct_body_set_priority", lib().mct_body_set_priority(self.h, 1 if high else 0))

    def close(self):
        if self.h:
            lib().mct_body_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def forward(self, ncells, points, params, locations, n0, n1):
        ncells = np.ascontiguousarray(ncells, np.int32)
        nch = ncells.size
        points = np.ascontiguousarray(points, np.float64)
        params = np.ascontiguousarray(params, np.float64)
        locations = np.ascontiguousarray(locations, np.float64).reshape(nch, self.nsrc, 4)
        n0 = np.ascontiguousarray(n0, np.float64).reshape(nch, self.np)
        n1 = np.ascontiguousarray(n1, np.float64).reshape(nch, self.np)
        out = np.zeros((nch, 4))
        check("mct_body_forward", lib().mct_body_forward(self.h, nch, ptr(ncells), ptr(points), ptr(params),
                                                         ptr(locations), ptr(n0), ptr(n1), ptr(out)))
        return out

    def location_likelihood(self, locations, n0, n1, times=False):
        """body_location_likelihood on the stored fields (settings dynamic=1):
        chains 0..nchains-1's committed fields read at the proposed event
        locations (nchains, nsrc, 4). Returns out (nchains, 4), and with
        times the interpolated times (nchains, np, nsrc*nrev)."""
        locations = np.ascontiguousarray(locations, np.float64)
        nch = locations.shape[0]
        locations = locations.reshape(nch, self.nsrc, 4)
        n0 = np.ascontiguousarray(n0, np.float64).reshape(nch, self.np)
        n1 = np.ascontiguousarray(n1, np.float64).reshape(nch, self.np)
        out = np.zeros((nch, 4))
        pt = np.zeros((nch, self.np, self.nsrc * self.nrev)) if times else None
        check("mct_body_location_likelihood",
              lib().mct_body_location_likelihood(self.h, nch, ptr(locations), ptr(n0), ptr(n1), ptr(out), ptr(pt)))
        return (out, pt) if times else out

    def location_commit(self, accept):
        accept = np.ascontiguousarray(accept, np.int32)
        check("mct_body_location_commit", lib().mct_body_location_commit(self.h, accept.size, ptr(accept)))

    def submit(self, ncells, points, params, locations, n0, n1):
        """Starts forward() on the context's worker thread without waiting;
        poll() collects it."""
        ncells = np.ascontiguousarray(ncells, np.int32)
        nch = ncells.size
        points = np.ascontiguousarray(points, np.float64)
        params = np.ascontiguousarray(params, np.float64)
        locations = np.ascontiguousarray(locations, np.float64).reshape(nch, self.nsrc, 4)
        n0 = np.ascontiguousarray(n0, np.float64).reshape(nch, self.np)
        n1 = np.ascontiguousarray(n1, np.float64).reshape(nch, self.np)
        check("mct_body_submit", lib().mct_body_submit(self.h, nch, ptr(ncells), ptr(points), ptr(params),
                                                       ptr(locations), ptr(n0), ptr(n1)))
        self._pending = nch

    def poll(self):
        """(done, out): out (nchains, 4) once the submitted batch finished."""
        out = np.zeros((self._pending, 4))
        done = ctypes.c_int()
        check("mct_body_poll", lib().mct_body_poll(self.h, ptr(out), ctypes.byref(done)))
        return bool(done.value), (out if done.value else None)

    def commit(self, accept):
        """Chains with accept[c] keep the last forward as their state."""
        accept = np.ascontiguousarray(accept, np.int32)
        check("mct_body_commit", lib().mct_body_commit(self.h, accept.size, ptr(accept)))

    def noise_likelihood(self, locations, n0, n1):
        """body_noise_likelihood: chains 0..nchains-1's committed travel times
        re-reduced with new noise parameters n0/n1 (nchains, np) and origin
        times (locations[..., 3]); no forward."""
        n0 = np.ascontiguousarray(n0, np.float64)
        nch = n0.shape[0]
        n0 = n0.reshape(nch, self.np)
        n1 = np.ascontiguousarray(n1, np.float64).reshape(nch, self.np)
        locations = np.ascontiguousarray(locations, np.float64).reshape(nch, self.nsrc, 4)
        out = np.zeros((nch, 4))
        check("mct_body_noise_likelihood",
              lib().mct_body_noise_likelihood(self.h, nch, ptr(locations), ptr(n0), ptr(n1), ptr(out)))
        return out

    def phase_time(self, index):
        pt = np.zeros((self.np, self.nsrc, self.nrev))
        passes = ctypes.c_int()
        check("mct_body_phase_time", lib().mct_body_phase_time(self.h, index, ptr(pt), ctypes.byref(passes)))
        return pt, passes.value
