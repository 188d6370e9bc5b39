"""GPU parity of the batched body-wave likelihood (gridding -> P/S 3D travel
times from the stations -> misfit with origin times) against the oracle's
composition of the reference path (kdtree gridding, the reference's own
fastMarching3D restated bit-exactly, the misfit)."""
import ctypes

import numpy as np
import pytest

from mctomo_gb300 import BodyLikelihood, synthetic

pytestmark = pytest.mark.gpu
EIK3_TILES, EIK3_HEAP = 0x10, 0x20
P = lambda a: None if a is None else a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
TT_TOL = {0: 1e-4, 1: 5e-2}   # tile solver, per order, see test_gpu_eik3


def oracle_body(orc, grid, settings, data, ev, n, pts, par, n0, n1):
    nx, ny, nz = grid["nx"], grid["ny"], grid["nz"]
    shp = (nx, ny, nz)
    sid = np.zeros(shp, np.int32); vp = np.zeros(shp); vs = np.zeros(shp); rho = np.zeros(shp)
    orc.orc_kdtree_to_grid(3, int(n), P(np.ascontiguousarray(pts[:n])), P(np.ascontiguousarray(par[:n])), nx, ny, nz,
                           grid["xmin"], grid["ymin"], grid["zmin"], grid["dx"], grid["dy"], grid["dz"], 1, nx, 1, ny,
                           1, nz, P(sid), P(vp), P(vs), P(rho))
    nsrc, rev, npp = data["nsrc"], np.asarray(data["rev"]), settings["np"]
    nrev = len(rev)
    dzs = grid["dz"] / grid["scaling"]; zms = grid["zmin"] / grid["scaling"]
    pt = np.zeros((npp, nsrc, nrev))
    locs = np.ascontiguousarray(ev[:, :3])
    for p, vel in enumerate([vp, vs][:npp]):
        for k in range(nrev):          # from the stations (events outnumber them)
            tt = np.zeros(nsrc)
            orc.orc_fast_marching3d(nx, ny, nz, grid["dx"], grid["dy"], dzs, grid["xmin"], grid["ymin"], zms,
                                    P(np.ascontiguousarray(vel)), P(np.ascontiguousarray(rev[k])), P(locs), nsrc,
                                    settings["order"], P(tt), None)
            pt[p, :, k] = tt
    return body_misfit(orc, settings, data, ev, pt, n0, n1), pt


def body_misfit(orc, settings, data, ev, pt, n0, n1):
    """The reference's misfit reduction (oracle) on the given phase times."""
    npp, nsrc, nrev = pt.shape
    npairs = nsrc * nrev
    dtt = np.zeros((npp, 3, npairs))
    dtt[:, 0] = data["ttime"]; dtt[:, 1] = data["sigma"]
    rs = np.zeros((npp, 2, npairs), np.int32); rs[:, 0] = data["raystat"]
    sig = np.zeros((npp, npairs)); out = np.zeros(3)
    ptf = np.ascontiguousarray(pt.reshape(npp, npairs))
    orc.orc_body_misfit(nsrc, nrev, npp, P(ptf), P(np.ascontiguousarray(ev[:, 3])), P(np.ascontiguousarray(dtt)),
                        P(np.ascontiguousarray(rs)), P(ptf), settings["sigdep"], P(np.ascontiguousarray(n0)),
                        P(np.ascontiguousarray(n1)), data["nrays"], P(sig), P(out))
    return out


@pytest.mark.parametrize("order,solver", [(0, 0), (1, 0), (0, EIK3_HEAP), (1, EIK3_TILES)])
def test_body_batch_matches_oracle(orc, gpulib, order, solver):
    rng = np.random.default_rng(40 + order)
    grid, settings, data, ev = synthetic.body_workload(rng, nx=31, ny=29, nz=17, extent=(15.0, 14.0, 8.0),
                                                      nevents=24, nstations=9)
    settings["order"] = order
    settings["solver"] = solver
    exact = solver == EIK3_HEAP or (solver == 0 and order == 1)   # the heap march
    lo = np.zeros(3); hi = np.array([15.0, 14.0, 8.0])
    nch, ncell_max = 3, 40
    ncells = np.array([12, 25, 40], np.int32)
    pts = np.zeros((nch, ncell_max, 3)); par = np.zeros((nch, ncell_max, 3))
    for c in range(nch):
        p, q = synthetic.voronoi_model_3d(rng, int(ncells[c]), lo, hi, (3.0 / 1.73, 7.5 / 1.73))
        q[:, 0] = q[:, 1] * 1.73
        pts[c, :ncells[c]] = p; par[c, :ncells[c]] = q
    locs = np.repeat(ev[None], nch, 0)
    n0 = np.zeros((nch, 2)); n1 = np.full((nch, 2), 0.05)
    lk = BodyLikelihood(grid, settings, data, nslots=nch, ncell_max=ncell_max)
    out = lk.forward(ncells, pts, par, locs, n0, n1)
    for c in range(nch):
        eo, ept = oracle_body(orc, grid, settings, data, ev, ncells[c], pts[c], par[c], n0[c], n1[c])
        pt, passes = lk.phase_time(c)
        if exact:
            assert passes == 0
            np.testing.assert_array_equal(pt, ept)
            # identical times: the likelihood equals the reference path's up
            # to the order of the misfit sums
            np.testing.assert_allclose(out[c, :3], eo, rtol=1e-12)
            continue
        assert passes > 0
        assert np.max(np.abs(pt - ept)) <= TT_TOL[order], np.max(np.abs(pt - ept))
        # the misfit reduction itself, on the GPU's own phase times
        np.testing.assert_allclose(out[c, :3], body_misfit(orc, settings, data, ev, pt, n0[c], n1[c]), rtol=1e-9)
        if order == 0:
            # end to end: times within 1e-4 s keep the likelihood close
            np.testing.assert_allclose(out[c, :3], eo, rtol=2e-3)
    lk.close()


@pytest.mark.parametrize("order,solver", [(0, EIK3_TILES), (1, EIK3_HEAP)])
def test_body_result_is_the_same_alone_and_in_the_mix(gpulib, order, solver):
    # the heap march is exact: a chain's times are the same bits alone and in
    # a call with other chains. The tile solver's fixed-point scale is chosen
    # per chain, and its relaxation order within a call varies with the
    # other chains' tiles, which moves the odd time by a few fixed-point
    # units (about 1e-8 s)
    rng = np.random.default_rng(48 + order)
    grid, settings, data, ev = synthetic.body_workload(rng, nx=31, ny=29, nz=17, extent=(15.0, 14.0, 8.0),
                                                      nevents=24, nstations=9)
    settings["order"] = order
    settings["solver"] = solver
    lo = np.zeros(3); hi = np.array([15.0, 14.0, 8.0])
    nch, ncell_max = 4, 40
    ncells = np.array([12, 25, 40, 7], np.int32)
    pts = np.zeros((nch, ncell_max, 3)); par = np.zeros((nch, ncell_max, 3))
    for c in range(nch):
        vr = (3.0 / 1.73, 7.5 / 1.73) if c != 2 else (1.0, 1.5)     # one slow chain
        p, q = synthetic.voronoi_model_3d(rng, int(ncells[c]), lo, hi, vr)
        q[:, 0] = q[:, 1] * 1.73
        pts[c, :ncells[c]] = p; par[c, :ncells[c]] = q
    locs = np.repeat(ev[None], nch, 0)
    n0 = np.zeros((nch, 2)); n1 = np.full((nch, 2), 0.05)
    mix = BodyLikelihood(grid, settings, data, nslots=nch, ncell_max=ncell_max)
    out = mix.forward(ncells, pts, par, locs, n0, n1)
    one = BodyLikelihood(grid, settings, data, nslots=1, ncell_max=ncell_max)
    for c in range(nch):
        o = one.forward(ncells[c:c + 1], pts[c:c + 1], par[c:c + 1], locs[:1], n0[:1], n1[:1])
        if solver == EIK3_HEAP:
            np.testing.assert_array_equal(o[0], out[c])
            np.testing.assert_array_equal(one.phase_time(0)[0], mix.phase_time(c)[0])
        else:
            assert o[0, 3] == out[c, 3]
            np.testing.assert_allclose(o[0, :3], out[c, :3], rtol=1e-8)
            np.testing.assert_allclose(one.phase_time(0)[0], mix.phase_time(c)[0], rtol=0, atol=1e-6)
    mix.close(); one.close()
