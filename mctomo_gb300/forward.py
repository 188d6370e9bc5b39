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


def modes_para(modetype, phase_group, tol=1e-6, dc=1e-3):
    """The reference surface likelihood's mode-search parameters
    (src/likelihood_surf.F90:173-182): tolmin = tol, tolmax = 10 tol, smin
    1e-3 / 5e-3 (single-precision literals) and every increment dc."""
    from ._lib import ModesPara
    return ModesPara(modetype, 1, phase_group, tol, 10 * tol, float(np.float32(1e-3)), float(np.float32(5e-3)),
                     dc, dc, dc, dc)


def surfmodes_para(thick, vp, vs, rho, freqs, paras):
    """surfmodes with explicit T_MODES_PARA (mct_surfmodes_para): columns with
    a low-velocity layer go to the generalized R/T search. Returns (phase,
    group, ierr)."""
    thick, vp, vs, rho, freqs = _f64(thick), _f64(vp), _f64(vs), _f64(rho), _f64(freqs)
    np_ = freqs.size
    phase = np.zeros(np_); group = np.zeros(np_)
    ierr = ctypes.c_int(0)
    rc = lib().mct_surfmodes_para(ptr(thick), ptr(vp), ptr(vs), ptr(rho), thick.size, ptr(freqs), np_,
                                  ctypes.byref(paras), ptr(phase), ptr(group), ctypes.byref(ierr))
    check("mct_surfmodes_para", rc)
    return phase, group, ierr.value


def surfmodes_route(nl, vp, vs, modetype):
    """surfmodes' routing per column (mct_surfmodes_route): 1 generalized
    R/T, 0 surfdisp96, -2 low-velocity layer under a fluid layer."""
    nl = np.ascontiguousarray(nl, dtype=np.int32)
    vp, vs = _f64(vp), _f64(vs)
    ncol, nl_max = vp.shape
    route = np.zeros(ncol, np.int32)
    check("mct_surfmodes_route", lib().mct_surfmodes_route(ncol, nl_max, ptr(nl), ptr(vp), ptr(vs), modetype,
                                                           ptr(route)))
    return route


def grt_batch(nl, thk, vp, vs, rho, freqs, paras):
    """The generalized R/T fundamental-mode search (RayleighModes / LoveModes,
    surfmodes/surfmodes.f90:185-303) for many FP64 columns: thk/vp/vs/rho
    (ncol, nl_max), nl (ncol,). Returns (phase, group, ierr, nevals) with
    phase/group shaped (ncol, np)."""
    nl = np.ascontiguousarray(nl, dtype=np.int32)
    thk, vp, vs, rho, freqs = _f64(thk), _f64(vp), _f64(vs), _f64(rho), _f64(freqs)
    ncol, nl_max = thk.shape
    np_ = freqs.size
    phase = np.zeros((ncol, np_)); group = np.zeros((ncol, np_))
    ierr = np.zeros(ncol, np.int32)
    cnt = ctypes.c_ulonglong(0)
    rc = lib().mct_grt_batch(ncol, nl_max, ptr(nl), ptr(thk), ptr(vp), ptr(vs), ptr(rho), np_, ptr(freqs),
                             ctypes.byref(paras), ptr(phase), ptr(group), ptr(ierr), ctypes.byref(cnt))
    check("mct_grt_batch", rc)
    return phase, group, ierr, cnt.value


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


def modrays(src, rev, srs, nvx, nvz, goxd, gozd, dvxd, dvzd, velv, gdx=1, gdz=1, asgr=1, sgdl=4,
            sgs=8, fom=1, snb=0.5, earth=6371.0, ttime=None, tfield=False):
    """fm2d modrays (fm2d/fm2dray_cartesian.f90:67-480) for travel times only
    (uar = 1). src: (nsrc, 2), rev: (nrc, 2), srs: (nsrc, nrc) path flags,
    velv: (nvx+2, nvz+2) C-order = Fortran (nvz+2, nvx+2). Returns ttime
    (nsrc, nrc) (C order = Fortran (nrc, nsrc)) and optionally the fields
    (nsrc, nnx, nnz)."""
    src = _f64(src); rev = _f64(rev)
    nsrc, nrc = src.shape[0], rev.shape[0]
    srsin = np.zeros(2 * nsrc * nrc, np.int32)
    srsin[:nsrc * nrc] = np.asarray(srs, np.int32).reshape(-1)
    velv = _f64(velv)
    assert velv.shape == (nvx + 2, nvz + 2)
    if ttime is None:
        ttime = np.zeros((nsrc, nrc))
    nnx = (nvx - 1) * gdx + 1
    nnz = (nvz - 1) * gdz + 1
    tf = np.zeros((nsrc, nnx, nnz)) if tfield else None
    cr = ctypes.c_int(0)
    sx, sz = np.ascontiguousarray(src[:, 0]), np.ascontiguousarray(src[:, 1])
    rx, rz = np.ascontiguousarray(rev[:, 0]), np.ascontiguousarray(rev[:, 1])
    rc = lib().mct_modrays(nsrc, ptr(sx), ptr(sz), nrc, ptr(rx), ptr(rz), ptr(srsin), 0, nvx, nvz,
                           goxd, gozd, dvxd, dvzd, ptr(velv), gdx, gdz, asgr, sgdl, sgs, earth, fom,
                           snb, ptr(ttime), 1, ctypes.byref(cr), ptr(tf))
    check("mct_modrays", rc)
    return (ttime, tf) if tfield else ttime


def modrays_batch(src, rev, srs, nvx, nvz, goxd, gozd, dvxd, dvzd, velv, gdx=1, gdz=1, asgr=1,
                  sgdl=4, sgs=8, fom=1, ttime=None, precision=0):
    """Many velocity maps with shared stations. velv: (nmaps, nvx+2, nvz+2);
    srs: (srs_nmaps, nsrc, nrc). Returns ttime (nmaps, nsrc, nrc)."""
    src = _f64(src); rev = _f64(rev); velv = _f64(velv)
    srs = np.ascontiguousarray(srs, np.int32)
    if srs.ndim == 2:
        srs = srs[None]
    nmaps = velv.shape[0]
    nsrc, nrc = src.shape[0], rev.shape[0]
    if ttime is None:
        ttime = np.zeros((nmaps, nsrc, nrc))
    sx, sz = np.ascontiguousarray(src[:, 0]), np.ascontiguousarray(src[:, 1])
    rx, rz = np.ascontiguousarray(rev[:, 0]), np.ascontiguousarray(rev[:, 1])
    rc = lib().mct_modrays_batch(nmaps, nsrc, ptr(sx), ptr(sz), nrc, ptr(rx), ptr(rz), srs.shape[0],
                                 ptr(srs), nvx, nvz, goxd, gozd, dvxd, dvzd, ptr(velv), gdx, gdz, asgr,
                                 sgdl, sgs, fom, ptr(ttime), None, int(precision))
    check("mct_modrays_batch", rc)
    return ttime


def modrays_group_batch(src, rev, srs, nvx, nvz, goxd, gozd, dvxd, dvzd, velv, gvel, gdx=1, gdz=1, asgr=1,
                        sgdl=4, sgs=8, fom=1, precision=0):
    """modrays with ray paths (uar = 0) and CalGroupTime on gvel (nmaps, nvx,
    nvz). Returns (phase times, group times, ray lengths), each (nmaps, nsrc,
    nrc), and the crazy-ray count per map."""
    src = _f64(src); rev = _f64(rev); velv = _f64(velv); gvel = _f64(gvel)
    srs = np.ascontiguousarray(srs, np.int32)
    if srs.ndim == 2:
        srs = srs[None]
    nmaps = velv.shape[0]
    nsrc, nrc = src.shape[0], rev.shape[0]
    tt = np.zeros((nmaps, nsrc, nrc)); gt = np.zeros_like(tt); ln = np.zeros_like(tt)
    crazy = np.zeros(nmaps, np.int32)
    sx, sz = np.ascontiguousarray(src[:, 0]), np.ascontiguousarray(src[:, 1])
    rx, rz = np.ascontiguousarray(rev[:, 0]), np.ascontiguousarray(rev[:, 1])
    rc = lib().mct_modrays_group_batch(nmaps, nsrc, ptr(sx), ptr(sz), nrc, ptr(rx), ptr(rz), srs.shape[0],
                                       ptr(srs), nvx, nvz, goxd, gozd, dvxd, dvzd, ptr(velv), ptr(gvel), gdx, gdz,
                                       asgr, sgdl, sgs, fom, ptr(tt), ptr(gt), ptr(ln), ptr(crazy), int(precision))
    check("mct_modrays_group_batch", rc)
    return tt, gt, ln, crazy


EIK3_TILES = 0x10
EIK3_HEAP = 0x20
_SOLVER = {None: 0, "tiles": EIK3_TILES, "heap": EIK3_HEAP}


def fast_marching3d(vel, h, lo, src, rev, order=1, tfield=False, solver=None):
    """fastMarching3D (fastmarching/fastMarching.cpp:26-129). vel: (nx, ny, nz)
    C order; h = (dx, dy, dz); lo = (xmin, ymin, zmin); src (3,); rev (nrev, 3).
    solver: None (heap march for order 1, tiles for order 0), "heap" or
    "tiles". Returns ttime (nrev,) and optionally the field (nx, ny, nz)."""
    order = int(order) | _SOLVER[solver]
    vel = _f64(vel)
    nx, ny, nz = vel.shape
    src = _f64(src); rev = _f64(rev).reshape(-1, 3)
    tt = np.zeros(rev.shape[0])
    tf = np.zeros_like(vel) if tfield else None
    rc = lib().mct_fast_marching3d(nx, ny, nz, float(h[0]), float(h[1]), float(h[2]), float(lo[0]), float(lo[1]),
                                   float(lo[2]), ptr(vel), ptr(src), ptr(rev), rev.shape[0], int(order), ptr(tt),
                                   ptr(tf))
    check("mct_fast_marching3d", rc)
    return (tt, tf) if tfield else tt


def eikonal3d_batch(vels, h, lo, solve_grid, srcs, rev, order=1, tfield=False, solver=None):
    """Many 3D solves: vels (ngrids, nx, ny, nz), solve_grid (nsolve,),
    srcs (nsolve, 3), shared receivers rev (nrev, 3); solver as for
    fast_marching3d. Returns ttime (nsolve, nrev), the optional fields and
    the number of tile passes (0 for the heap march)."""
    order = int(order) | _SOLVER[solver]
    vels = _f64(vels)
    ng, nx, ny, nz = vels.shape
    solve_grid = np.ascontiguousarray(solve_grid, np.int32)
    srcs = _f64(srcs).reshape(-1, 3)
    rev = _f64(rev).reshape(-1, 3)
    ns = srcs.shape[0]
    tt = np.zeros((ns, rev.shape[0]))
    tf = np.zeros((ns, nx, ny, nz)) if tfield else None
    passes = ctypes.c_int(0)
    rc = lib().mct_eikonal3d_batch(ns, nx, ny, nz, float(h[0]), float(h[1]), float(h[2]), float(lo[0]),
                                   float(lo[1]), float(lo[2]), ng, ptr(vels), ptr(solve_grid), ptr(srcs),
                                   rev.shape[0], ptr(rev), int(order), ptr(tt), ptr(tf), ctypes.byref(passes))
    check("mct_eikonal3d_batch", rc)
    return tt, tf, passes.value
