"""Python mirror of the reference's forward-modelling routines.

Each function keeps the reference routine's name, argument meaning and
Fortran array layout, and calls the CUDA library through the C ABI.
"""
import ctypes

import numpy as np

from ._lib import check, lib, ptr


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def kdtree_to_grid(points, params, nx, ny, nz, grid_lo, grid_step, box=None,
                   sites_id=None, vp=None, vs=None, rho=None):
    """Nearest-nucleus map of kdtree_to_grid (src/mcmc_loc2.f90:2002-2082;
    2D: mcmc2d/mcmc.f90:1469-1525).

    points: (n, d) nucleus coordinates (row i = RTI%points(:,i)); params:
    (n, 3) = (vp, vs, rho). Returns (sites_id, vp, vs, rho) shaped (nx, ny, nz)
    (C order, i.e. Fortran (nz,ny,nx)); for d=2 shaped (nx, ny).
    Existing output arrays may be passed to keep values outside ``box``.
    """
    points = _f64(points)
    params = _f64(params)
    n, d = points.shape
    shape = (nx, ny, nz) if d == 3 else (nx, ny)
    if sites_id is None:
        sites_id = np.zeros(shape, np.int32)
    if vp is None:
        vp = np.zeros(shape); vs = np.zeros(shape); rho = np.zeros(shape)
    lo = _f64(grid_lo)
    st = _f64(grid_step)
    b = None if box is None else np.ascontiguousarray(box, dtype=np.int32)
    rc = lib().mct_kdtree_to_grid(d, n, ptr(points), ptr(params), nx, ny, nz if d == 3 else 1,
                                  ptr(lo), ptr(st), ptr(b), ptr(sites_id), ptr(vp), ptr(vs), ptr(rho))
    check("mct_kdtree_to_grid", rc)
    return sites_id, vp, vs, rho


def surfdisp96(thkm, vpm, vsm, rhom, iwave, igr, t, dphase, mode=1, iflsph=0):
    """surfdisp96 (surfmodes/surfdisp96.f:52-382). Returns (cp, cg, ierr)."""
    thkm, vpm, vsm, rhom = _f32(thkm), _f32(vpm), _f32(vsm), _f32(rhom)
    t = _f64(t)
    kmax = t.size
    cp = np.zeros(kmax); cg = np.zeros(kmax)
    ierr = ctypes.c_int(0)
    rc = lib().mct_surfdisp96(ptr(thkm), ptr(vpm), ptr(vsm), ptr(rhom), thkm.size, iflsph, iwave,
                              mode, igr, kmax, ptr(t), float(dphase), ptr(cp), ptr(cg), ctypes.byref(ierr))
    check("mct_surfdisp96", rc)
    return cp, cg, ierr.value


def surfdisp_mmodes(thkm, vpm, vsm, rhom, iwave, mode, igr, t, dphase, iflsph=0):
    """surfdisp_mmodes (surfdisp96.f:385-701). cp/cg shaped (mode, kmax)."""
    thkm, vpm, vsm, rhom = _f32(thkm), _f32(vpm), _f32(vsm), _f32(rhom)
    t = _f64(t)
    kmax = t.size
    cp = np.zeros((mode, kmax)); cg = np.zeros((mode, kmax))
    ierr = ctypes.c_int(0)
    rc = lib().mct_surfdisp_mmodes(ptr(thkm), ptr(vpm), ptr(vsm), ptr(rhom), thkm.size, iflsph,
                                   iwave, mode, igr, kmax, ptr(t), float(dphase), ptr(cp), ptr(cg),
                                   ctypes.byref(ierr))
    check("mct_surfdisp_mmodes", rc)
    return cp, cg, ierr.value


def surfmodes(thick, vp, vs, rho, freqs, modetype, phase_group, dc):
    """surfmodes (surfmodes/surfmodes.f90:39-108). Returns (phase, group, ierr)."""
    thick, vp, vs, rho, freqs = _f64(thick), _f64(vp), _f64(vs), _f64(rho), _f64(freqs)
    np_ = freqs.size
    phase = np.zeros(np_); group = np.zeros(np_)
    ierr = ctypes.c_int(0)
    rc = lib().mct_surfmodes(ptr(thick), ptr(vp), ptr(vs), ptr(rho), thick.size, ptr(freqs), np_,
                             modetype, phase_group, float(dc), ptr(phase), ptr(group), ctypes.byref(ierr))
    check("mct_surfmodes", rc)
    return phase, group, ierr.value


def surfdisp_batch(nl, thk, vp, vs, rho, periods, iwave, igr, dphase, mode=1, multimode=False,
                   precision=0):
    """Many columns at once. thk/vp/vs/rho: (ncol, nl_max) REAL*4 models, nl:
    (ncol,) layer counts. Returns (cp, cg, ierr, (n_fp64, n_fp32)) with cp/cg
    shaped (ncol, mode, np)."""
    nl = np.ascontiguousarray(nl, dtype=np.int32)
    thk, vp, vs, rho = _f32(thk), _f32(vp), _f32(vs), _f32(rho)
    periods = _f64(periods)
    ncol, nl_max = thk.shape
    np_ = periods.size
    cp = np.zeros((ncol, mode, np_)); cg = np.zeros((ncol, mode, np_))
    ierr = np.zeros(ncol, np.int32)
    cnt = (ctypes.c_ulonglong * 2)()
    rc = lib().mct_surfdisp_batch(ncol, nl_max, ptr(nl), ptr(thk), ptr(vp), ptr(vs), ptr(rho), np_,
                                  ptr(periods), iwave, mode, igr, float(dphase), int(multimode),
                                  int(precision), ptr(cp), ptr(cg), ptr(ierr), cnt)
    check("mct_surfdisp_batch", rc)
    return cp, cg, ierr, (cnt[0], cnt[1])
