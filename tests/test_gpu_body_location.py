"""GPU: the body-wave location step on stored travel-time fields
(settings dynamic = 1, the reference's body_location_likelihood,
src/likelihood_body.F90:82-149): the committed fields (the exact heap march,
one per station and phase) read at proposed event locations give the
oracle's Interpolate3d times bit for bit on the oracle's own fields, and the
misfit; accepted location steps become the committed times; a context
without stored fields refuses the step."""
import ctypes

import numpy as np
import pytest

from mctomo_gb300 import BodyLikelihood, MctError, synthetic
from oracle import location as oloc
from test_gpu_body import body_misfit

pytestmark = pytest.mark.gpu
EIK3_HEAP = 0x20
P = lambda a: None if a is None else a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731


def case(seed, dynamic=1):
    rng = np.random.default_rng(seed)
    grid, settings, data, ev = synthetic.body_workload(rng, nx=23, ny=21, nz=13, extent=(11.0, 10.0, 6.0),
                                                      nevents=18, nstations=7)
    settings.update(order=1, solver=EIK3_HEAP, dynamic=dynamic, sigdep=1)
    lo = np.zeros(3); hi = np.array([11.0, 10.0, 6.0])
    nch, ncell_max = 2, 20
    ncells = np.array([9, 16], np.int32)
    pts = np.zeros((nch, ncell_max, 3)); par = np.zeros((nch, ncell_max, 3))
    for c in range(nch):
        p, q = synthetic.voronoi_model_3d(rng, int(ncells[c]), lo, hi, (3.0 / 1.73, 7.5 / 1.73))
        q[:, 0] = q[:, 1] * 1.73
        pts[c, :ncells[c]] = p; par[c, :ncells[c]] = q
    return rng, grid, settings, data, ev, ncells, pts, par


def oracle_fields(orc, grid, data, n, pts, par):
    nx, ny, nz = grid["nx"], grid["ny"], grid["nz"]
    shp = (nx, ny, nz)
    sid = np.zeros(shp, np.int32); vp = np.zeros(shp); vs = np.zeros(shp); rho = np.zeros(shp)
    orc.orc_kdtree_to_grid(3, int(n), P(np.ascontiguousarray(pts[:n])), P(np.ascontiguousarray(par[:n])), nx, ny, nz,
                           grid["xmin"], grid["ymin"], grid["zmin"], grid["dx"], grid["dy"], grid["dz"], 1, nx, 1, ny,
                           1, nz, P(sid), P(vp), P(vs), P(rho))
    rev = np.asarray(data["rev"])
    dzs, zms = grid["dz"] / grid["scaling"], grid["zmin"] / grid["scaling"]
    fields = []
    for vel in (vp, vs):
        fp = []
        for k in range(len(rev)):
            tt, tf = np.zeros(1), np.zeros(shp)
            orc.orc_fast_marching3d(nx, ny, nz, grid["dx"], grid["dy"], dzs, grid["xmin"], grid["ymin"], zms,
                                    P(np.ascontiguousarray(vel)), P(np.ascontiguousarray(rev[k])),
                                    P(np.ascontiguousarray(rev[k])), 1, 1, P(tt), P(tf))
            fp.append(tf)
        fields.append(fp)
    return fields


def test_location_step_reads_the_committed_fields(orc, gpulib):
    rng, grid, settings, data, ev, ncells, pts, par = case(81)
    nsrc, nrev = data["nsrc"], len(data["rev"])
    lk = BodyLikelihood(grid, settings, data, nslots=2, ncell_max=20)
    locs = np.repeat(ev[None], 2, 0)
    n0, n1 = np.full((2, 2), 0.01), np.full((2, 2), 0.03)
    # nothing committed yet
    assert np.all(lk.location_likelihood(locs, n0, n1)[:, 3] == 16)
    lk.forward(ncells, pts, par, locs, n0, n1)
    lk.commit(np.ones(2, np.int32))
    # proposed locations: every event moved, some to the grid's faces
    new = locs.copy()
    new[:, :, :3] += rng.normal(0, 0.4, (2, nsrc, 3))
    for a, hi in enumerate((11.0, 10.0, 6.0)):
        new[:, :, a] = np.clip(new[:, :, a], 0.0, hi)
    new[0, 0, :3] = [11.0, 10.0, 6.0]
    out, times = lk.location_likelihood(new, n0, n1, times=True)
    assert np.all(out[:, 3] == 0)
    for c in range(2):
        fields = oracle_fields(orc, grid, data, ncells[c], pts[c], par[c])
        exp = np.zeros((2, nsrc, nrev))
        for p in range(2):
            for j in range(nsrc):
                for k in range(nrev):
                    exp[p, j, k] = oloc.interpolate3d(fields[p][k], grid, new[c, j, :3])
        np.testing.assert_array_equal(times[c].reshape(2, nsrc, nrev), exp)
        # the oracle's C read-out (the CPU path the bench times) agrees
        ct = np.zeros((2, nsrc, nrev))
        orc.orc_location_times(grid["nx"], grid["ny"], grid["nz"], grid["xmin"], grid["ymin"], grid["zmin"],
                               grid["dx"], grid["dy"], grid["dz"], grid["scaling"], 2, nsrc, nrev,
                               P(np.ascontiguousarray(np.stack([np.stack(f) for f in fields]))),
                               P(np.ascontiguousarray(new[c])), P(ct))
        np.testing.assert_array_equal(ct, exp)
        eo = body_misfit(orc, dict(settings, sigdep=1), data, new[c], exp, n0[c], n1[c])
        np.testing.assert_allclose(out[c, :3], eo, rtol=1e-12)
    # chain 0 accepts its location step: its committed times are now the
    # interpolated ones, which the noise-only likelihood re-reduces
    lk.location_commit(np.array([1, 0], np.int32))
    nl = lk.noise_likelihood(new, n0, n1)
    assert nl[0, 0] == out[0, 0]
    lk.close()


def test_location_step_needs_stored_fields(gpulib):
    _, grid, settings, data, ev, ncells, pts, par = case(82, dynamic=0)
    lk = BodyLikelihood(grid, settings, data, nslots=2, ncell_max=20)
    with pytest.raises(MctError):
        lk.location_likelihood(np.repeat(ev[None], 2, 0), np.zeros((2, 2)), np.zeros((2, 2)))
    lk.close()
