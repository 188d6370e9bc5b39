"""Surface-wave likelihood with device-resident chains (C ABI mct_surf_*).

Mirrors the reference's likelihood() for datatype 2
(src/likelihood.f90:57-93 -> src/likelihood_surf.F90:110-410) evaluated for
many chains at once; ``forward`` is the proposal evaluation, ``commit`` the
sampler's accept (a chain that is not committed keeps its previous state,
the reject path).
"""
import ctypes

import numpy as np

from ._lib import check, lib, ptr

LAW_EXPLICIT, LAW_REFERENCE, LAW_FIXED_RHO = 0, 1, 2


class Grid(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
                ("xmin", ctypes.c_double), ("ymin", ctypes.c_double), ("zmin", ctypes.c_double),
                ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("dz", ctypes.c_double),
                ("scaling", ctypes.c_double), ("water_depth", ctypes.c_double)]


class SurfSettings(ctypes.Structure):
    _fields_ = [("raylov", ctypes.c_int), ("phase_group", ctypes.c_int), ("dphase", ctypes.c_double),
                ("gridx", ctypes.c_int), ("gridy", ctypes.c_int), ("sgref", ctypes.c_int),
                ("sgdic", ctypes.c_int), ("sgext", ctypes.c_int), ("order", ctypes.c_int),
                ("sigdep", ctypes.c_int), ("material_law", ctypes.c_int), ("rho_value", ctypes.c_double),
                ("precision", ctypes.c_int), ("tt_precision", ctypes.c_int), ("straight", ctypes.c_int)]


class SurfData(ctypes.Structure):
    _fields_ = [("nsrc", ctypes.c_int), ("nrev", ctypes.c_int), ("np", ctypes.c_int),
                ("src", ctypes.c_void_p), ("rev", ctypes.c_void_p), ("freqs", ctypes.c_void_p),
                ("raystat", ctypes.c_void_p), ("ttime", ctypes.c_void_p), ("sigma", ctypes.c_void_p),
                ("nrays", ctypes.c_int)]


def _structs(grid, settings, data):
    g = Grid(**grid)
    s = SurfSettings(**settings)
    npd = len(data["freqs"])
    arrs = {k: np.ascontiguousarray(data[k], np.float64) for k in ("src", "rev", "freqs", "ttime")}
    arrs["raystat"] = np.ascontiguousarray(data["raystat"], np.int32)
    sig = data.get("sigma")
    arrs["sigma"] = None if sig is None else np.ascontiguousarray(sig, np.float64)
    d = SurfData(len(arrs["src"]), len(arrs["rev"]), npd, arrs["src"].ctypes.data,
                 arrs["rev"].ctypes.data, arrs["freqs"].ctypes.data, arrs["raystat"].ctypes.data,
                 arrs["ttime"].ctypes.data, None if arrs["sigma"] is None else arrs["sigma"].ctypes.data,
                 int(data.get("nrays", int((arrs["raystat"] == 1).sum()))))
    return g, s, d, arrs


def device_bytes(grid, settings, data, nslots, ncell_max):
    """Device memory a SurfaceLikelihood with these arguments allocates."""
    g, s, d, _keep = _structs(grid, settings, data)
    out = ctypes.c_size_t()
    check("mct_surf_device_bytes", lib().mct_surf_device_bytes(ctypes.byref(g), ctypes.byref(s), ctypes.byref(d),
                                                               nslots, ncell_max, ctypes.byref(out)))
    return out.value


class SurfaceLikelihood:
    """grid: dict with nx, ny, nz, xmin, ymin, zmin, dx, dy, dz, scaling,
    water_depth. settings: dict of mct_surf_settings fields. data: dict with
    src (nsrc,2), rev (nrev,2), freqs (np,), raystat (np, nsrc*nrev),
    ttime (np, nsrc*nrev), optional sigma (np, nsrc*nrev)."""

    def __init__(self, grid, settings, data, nslots, ncell_max):
        self._keep = []
        g, s, d, arrs = _structs(grid, settings, data)
        self.np = len(data["freqs"])
        self._keep.append(arrs)
        self.nsrc, self.nrev = d.nsrc, d.nrev
        self.nslots, self.ncell_max = nslots, ncell_max
        self.nx, self.ny, self.nz = g.nx, g.ny, g.nz
        h = ctypes.c_void_p()
        check("mct_surf_create", lib().mct_surf_create(ctypes.byref(g), ctypes.byref(s), ctypes.byref(d),
                                                       nslots, ncell_max, ctypes.byref(h)))
        self.h = h

    def set_priority(self, high):
        """Run this context's work on a high-priority (True) or a normal
        stream of the device."""
        check("mct_surf_set_priority", lib().mct_surf_set_priority(self.h, 1 if high else 0))

    def set_sm_share(self, share):
        """Keep this context's 2D travel-time kernels to a share (0-1) of the
        device's SMs (0 or 1: all of them); results do not depend on it."""
        check("mct_surf_set_sm_share", lib().mct_surf_set_sm_share(self.h, float(share)))

    def close(self):
        if self.h:
            lib().mct_surf_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def forward(self, slots, ncells, points, params, n0, n1):
        """points/params: (nchains, ncell_max, 3); n0/n1: (nchains, np).
        Returns out (nchains, 4) = like, misfit, unweighted misfit, status."""
        slots = np.ascontiguousarray(slots, np.int32)
        nch = slots.size
        ncells = np.ascontiguousarray(ncells, np.int32)
        points = np.ascontiguousarray(points, np.float64)
        params = np.ascontiguousarray(params, np.float64)
        assert points.shape == (nch, self.ncell_max, 3) and params.shape == points.shape
        n0 = np.ascontiguousarray(n0, np.float64).reshape(nch, self.np)
        n1 = np.ascontiguousarray(n1, np.float64).reshape(nch, self.np)
        out = np.zeros((nch, 4))
        check("mct_surf_forward", lib().mct_surf_forward(self.h, nch, ptr(slots), ptr(ncells), ptr(points),
                                                         ptr(params), ptr(n0), ptr(n1), ptr(out)))
        return out

    def submit(self, slots, ncells, points, params, n0, n1):
        """Starts forward() without waiting; poll() collects it."""
        slots = np.ascontiguousarray(slots, np.int32)
        nch = slots.size
        ncells = np.ascontiguousarray(ncells, np.int32)
        points = np.ascontiguousarray(points, np.float64)
        params = np.ascontiguousarray(params, np.float64)
        n0 = np.ascontiguousarray(n0, np.float64).reshape(nch, self.np)
        n1 = np.ascontiguousarray(n1, np.float64).reshape(nch, self.np)
        check("mct_surf_submit", lib().mct_surf_submit(self.h, nch, ptr(slots), ptr(ncells), ptr(points),
                                                       ptr(params), ptr(n0), ptr(n1)))
        self._pending = nch

    def poll(self):
        """(done, out): out (nchains, 4) once the submitted batch finished."""
        out = np.zeros((self._pending, 4))
        done = ctypes.c_int()
        check("mct_surf_poll", lib().mct_surf_poll(self.h, ptr(out), ctypes.byref(done)))
        return bool(done.value), (out if done.value else None)

    def stat_add(self, slots):
        """stat_rti on the device: add each slot's committed model to its
        posterior sums (vp, vp^2, vs, vs^2 per node)."""
        slots = np.ascontiguousarray(slots, np.int32)
        check("mct_surf_stat_add", lib().mct_surf_stat_add(self.h, slots.size, ptr(slots)))

    def stat_read(self, slot):
        """(mean_vp, mean_vs, msq_vp, msq_vs, nthin): each (nx, ny, nz), the
        sums over the number of models added (write_mean / write_var)."""
        shape = (self.nx, self.ny, self.nz)
        mp, ms, qp, qs = (np.zeros(shape) for _ in range(4))
        n = ctypes.c_int()
        check("mct_surf_stat_read", lib().mct_surf_stat_read(self.h, int(slot), ptr(mp), ptr(ms), ptr(qp), ptr(qs),
                                                             ctypes.byref(n)))
        return mp, ms, qp, qs, n.value

    def stat_reset(self, slot):
        check("mct_surf_stat_reset", lib().mct_surf_stat_reset(self.h, int(slot)))

    def admit(self):
        """Claims a free chain slot (MctError when none is free)."""
        slot = ctypes.c_int()
        check("mct_surf_admit", lib().mct_surf_admit(self.h, ctypes.byref(slot)))
        return slot.value

    def evict(self, slot):
        check("mct_surf_evict", lib().mct_surf_evict(self.h, int(slot)))

    def commit(self, accept):
        accept = np.ascontiguousarray(accept, np.int32)
        check("mct_surf_commit", lib().mct_surf_commit(self.h, ptr(accept)))

    def noise_likelihood(self, slots, n0, n1):
        """surf_noise_likelihood: the committed travel times of each slot
        re-reduced with new noise parameters n0/n1 (nchains, np); no forward.
        Returns out (nchains, 4) as forward."""
        slots = np.ascontiguousarray(slots, np.int32)
        nch = slots.size
        n0 = np.ascontiguousarray(n0, np.float64).reshape(nch, self.np)
        n1 = np.ascontiguousarray(n1, np.float64).reshape(nch, self.np)
        out = np.zeros((nch, 4))
        check("mct_surf_noise_likelihood",
              lib().mct_surf_noise_likelihood(self.h, nch, ptr(slots), ptr(n0), ptr(n1), ptr(out)))
        return out

    def phase_time(self, index):
        """Last forward's travel times (np, nsrc, nrev) and phase maps (np, nx, ny)."""
        pt = np.zeros((self.np, self.nsrc, self.nrev))
        pv = np.zeros((self.np, self.nx, self.ny))
        check("mct_surf_phase_time", lib().mct_surf_phase_time(self.h, index, ptr(pt), ptr(pv)))
        return pt, pv
