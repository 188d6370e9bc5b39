"""GPU parity of the noise-only likelihoods (surf_noise_likelihood,
body_noise_likelihood): the kept travel times re-reduced with new noise
parameters, against the oracle's restatement of the reduction on the same
travel times, and the surface version's use of the committed (not the last
proposed) state."""
import ctypes

import numpy as np
import pytest

from mctomo_gb300 import BodyLikelihood, SurfaceLikelihood, synthetic

pytestmark = pytest.mark.gpu
P = lambda a: None if a is None else a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
RTOL = 1e-9


def surf_oracle(orc, data, pt, n0, n1):
    npd, nsrc, nrev = pt.shape
    npairs = nsrc * nrev
    dtt = np.zeros((npd, 3, npairs)); dtt[:, 0] = np.asarray(data["ttime"]).reshape(npd, npairs)
    rs = np.zeros((npd, 2, npairs), np.int32); rs[:, 0] = np.asarray(data["raystat"]).reshape(npd, npairs)
    ptf = np.ascontiguousarray(pt.reshape(npd, npairs))
    sig = np.zeros((npd, npairs)); out = np.zeros(3)
    st = orc.orc_surf_misfit(nsrc, nrev, npd, P(ptf), P(dtt), P(rs), P(ptf), 1, P(np.ascontiguousarray(n0)),
                             P(np.ascontiguousarray(n1)), data["nrays"], P(sig), P(out))
    return out, st


def test_surface_noise_likelihood_uses_committed_times(orc, gpulib):
    rng = np.random.default_rng(31)
    grid, settings, data = synthetic.surface_workload(rng, nx=21, ny=19, nz=11, extent=(20.0, 18.0, 3.0),
                                                      nstations=9, nperiods=5, pmin=0.5, pmax=3.0)
    nch, ncell_max = 3, 40
    ncells, pts, par = synthetic.surface_chain_models(rng, nch, ncell_max, grid, ncell_range=(6, ncell_max))
    npd = len(data["freqs"])
    lk = SurfaceLikelihood(grid, settings, data, nslots=nch, ncell_max=ncell_max)
    n0 = np.full((nch, npd), 0.02); n1 = np.full((nch, npd), 0.01)
    slots = np.arange(nch)
    lk.forward(slots, ncells, pts, par, n0, n1)
    committed = [lk.phase_time(c)[0] for c in range(nch)]
    lk.commit(np.ones(nch, np.int32))
    # a second proposal, rejected for chain 1: its noise likelihood must
    # still use the first model's times
    pts2, par2 = synthetic.perturb_chain_models(rng, ncells, pts, par, grid)
    lk.forward(slots, ncells, pts2, par2, n0, n1)
    second = [lk.phase_time(c)[0] for c in range(nch)]
    lk.commit(np.array([1, 0, 1], np.int32))
    committed = [second[0], committed[1], second[2]]
    m0 = rng.uniform(0.005, 0.05, (nch, npd)); m1 = rng.uniform(0.0, 0.05, (nch, npd))
    got = lk.noise_likelihood(slots, m0, m1)
    for c in range(nch):
        exp, st = surf_oracle(orc, data, committed[c], m0[c], m1[c])
        assert st == 0 and got[c, 3] == 0
        np.testing.assert_allclose(got[c, :3], exp, rtol=RTOL)
    # a subset in any order
    sub = lk.noise_likelihood(np.array([2, 0]), m0[[2, 0]], m1[[2, 0]])
    np.testing.assert_allclose(sub, got[[2, 0]], rtol=RTOL)
    lk.close()


def test_surface_noise_likelihood_zero_sigma_and_empty_slot(gpulib):
    rng = np.random.default_rng(32)
    grid, settings, data = synthetic.surface_workload(rng, nx=21, ny=19, nz=11, extent=(20.0, 18.0, 3.0),
                                                      nstations=6, nperiods=3, pmin=0.5, pmax=3.0)
    ncells, pts, par = synthetic.surface_chain_models(rng, 2, 20, grid, ncell_range=(6, 20))
    npd = len(data["freqs"])
    lk = SurfaceLikelihood(grid, settings, data, nslots=3, ncell_max=20)
    n0 = np.full((2, npd), 0.02); n1 = np.full((2, npd), 0.01)
    lk.forward(np.arange(2), ncells, pts, par, n0, n1)
    lk.commit(np.ones(2, np.int32))
    out = lk.noise_likelihood(np.array([0, 2]), np.zeros((2, npd)), np.zeros((2, npd)))
    assert int(out[0, 3]) & 8          # zero sigma: the reference's fatal error
    assert int(out[1, 3]) & 16         # slot 2 never committed
    assert np.all(out[:, 0] > 1e300)
    lk.close()


def test_body_noise_likelihood_matches_oracle(orc, gpulib):
    rng = np.random.default_rng(33)
    grid, settings, data, ev = synthetic.body_workload(rng, nx=25, ny=23, nz=13, extent=(12.0, 11.0, 6.0),
                                                      nevents=14, nstations=6)
    settings["order"] = 0
    nch, ncell_max = 2, 30
    lo = np.zeros(3); hi = np.array([12.0, 11.0, 6.0])
    ncells = np.array([10, 30], np.int32)
    pts = np.zeros((nch, ncell_max, 3)); par = np.zeros((nch, ncell_max, 3))
    for c in range(nch):
        p, q = synthetic.voronoi_model_3d(rng, int(ncells[c]), lo, hi, (3.0 / 1.73, 7.5 / 1.73))
        q[:, 0] = q[:, 1] * 1.73
        pts[c, :ncells[c]] = p; par[c, :ncells[c]] = q
    lk = BodyLikelihood(grid, settings, data, nslots=nch, ncell_max=ncell_max)
    locs = np.repeat(ev[None], nch, 0)
    lk.forward(ncells, pts, par, locs, np.zeros((nch, 2)), np.full((nch, 2), 0.05))
    m0 = np.array([[0.01, 0.02], [0.0, 0.03]]); m1 = np.array([[0.04, 0.05], [0.06, 0.02]])
    locs2 = locs.copy(); locs2[:, :, 3] += rng.uniform(-0.2, 0.2, (nch, locs.shape[1]))
    assert np.all(lk.noise_likelihood(locs2, m0, m1)[:, 3] == 16)    # nothing committed yet
    lk.commit(np.ones(nch, np.int32))
    committed = [lk.phase_time(c)[0] for c in range(nch)]
    # a rejected proposal leaves the committed times
    lk.forward(ncells, pts, par * 1.05, locs, np.zeros((nch, 2)), np.full((nch, 2), 0.05))
    lk.commit(np.zeros(nch, np.int32))
    got = lk.noise_likelihood(locs2, m0, m1)
    nsrc, nrev = data["nsrc"], len(data["rev"])
    npairs = nsrc * nrev
    for c in range(nch):
        pt = committed[c]
        dtt = np.zeros((2, 3, npairs)); dtt[:, 0] = data["ttime"]; dtt[:, 1] = data["sigma"]
        rs = np.zeros((2, 2, npairs), np.int32); rs[:, 0] = data["raystat"]
        ptf = np.ascontiguousarray(pt.reshape(2, npairs))
        sig = np.zeros((2, npairs)); exp = np.zeros(3)
        orc.orc_body_misfit(nsrc, nrev, 2, P(ptf), P(np.ascontiguousarray(locs2[c, :, 3])), P(dtt), P(rs), P(ptf), 1,
                            P(np.ascontiguousarray(m0[c])), P(np.ascontiguousarray(m1[c])), data["nrays"], P(sig),
                            P(exp))
        np.testing.assert_allclose(got[c, :3], exp, rtol=RTOL)
    lk.close()
