"""GPU: mct_tt2d_submit/poll and mct_body_submit/poll give the results of
the blocking forward (same bits; the body context here runs the exact heap
march), refuse the context's other calls until the batch is polled, let one
host thread keep several contexts busy, and a body context can be destroyed
with a batch in flight."""
import time

import numpy as np
import pytest

from mctomo_gb300 import BodyLikelihood, MctError, TravelTime2DLikelihood, synthetic

pytestmark = pytest.mark.gpu
EIK3_HEAP = 0x20


def wait(lk, limit=120.0):
    t0 = time.time()
    done, out = lk.poll()
    while not done:
        assert time.time() - t0 < limit, "batch did not finish"
        time.sleep(0.001)
        done, out = lk.poll()
    return out


def tt2d_case(seed, nch=4):
    rng = np.random.default_rng(seed)
    g, s, d = synthetic.tt2d_workload(rng, nx=41, ny=41, nstations=12)
    nc, pts, par = synthetic.tt2d_chain_models(rng, nch, 40, g, (4, 40))
    return g, s, d, nc, pts, par, np.zeros((nch, 2)), np.full((nch, 2), 0.05)


def body_case(seed, nch=3):
    rng = np.random.default_rng(seed)
    g, s, d, ev = synthetic.body_workload(rng, nx=31, ny=29, nz=17, extent=(15.0, 14.0, 8.0), nevents=24,
                                          nstations=9)
    s["order"] = 1
    s["solver"] = EIK3_HEAP
    lo = np.zeros(3); hi = np.array([15.0, 14.0, 8.0])
    nc = np.array([12, 25, 7][:nch], np.int32)
    pts = np.zeros((nch, 30, 3)); par = np.zeros((nch, 30, 3))
    for c in range(nch):
        p, q = synthetic.voronoi_model_3d(rng, int(nc[c]), lo, hi, (3.0 / 1.73, 7.5 / 1.73))
        q[:, 0] = q[:, 1] * 1.73
        pts[c, :nc[c]] = p; par[c, :nc[c]] = q
    locs = np.repeat(ev[None], nch, 0)
    return g, s, d, nc, pts, par, locs, np.zeros((nch, 2)), np.full((nch, 2), 0.05)


def test_tt2d_submit_poll_matches_forward(gpulib):
    g, s, d, nc, pts, par, n0, n1 = tt2d_case(61)
    lk = TravelTime2DLikelihood(g, s, d, nslots=4, ncell_max=40)
    ref = lk.forward(nc, pts, par, n0, n1)
    pt = [lk.phase_time(i) for i in range(4)]
    lk.submit(nc, pts, par, n0, n1)
    with pytest.raises(MctError):
        lk.forward(nc, pts, par, n0, n1)
    with pytest.raises(MctError):
        lk.commit(np.ones(4, np.int32))
    with pytest.raises(MctError):
        lk.submit(nc, pts, par, n0, n1)
    out = wait(lk)
    assert np.array_equal(out, ref)
    for i in range(4):
        assert np.array_equal(lk.phase_time(i), pt[i])
    # commit applies to the polled batch; noise-only results follow it
    lk.commit(np.array([1, 0, 1, 1], np.int32))
    nl = lk.noise_likelihood(n0, n1)
    assert np.all(nl[[0, 2, 3], 3] == 0) and nl[1, 3] == 16     # chain 1 has nothing committed
    np.testing.assert_allclose(nl[[0, 2, 3], 0], ref[[0, 2, 3], 0], rtol=1e-12)
    # poll with nothing submitted is an argument error
    with pytest.raises(MctError):
        lk.poll()
    lk.close()


def test_body_submit_poll_matches_forward(gpulib):
    g, s, d, nc, pts, par, locs, n0, n1 = body_case(62)
    lk = BodyLikelihood(g, s, d, nslots=3, ncell_max=30)
    ref = lk.forward(nc, pts, par, locs, n0, n1)
    pt = [lk.phase_time(i)[0] for i in range(3)]
    lk.submit(nc, pts, par, locs, n0, n1)
    with pytest.raises(MctError):
        lk.forward(nc, pts, par, locs, n0, n1)
    with pytest.raises(MctError):
        lk.submit(nc, pts, par, locs, n0, n1)
    out = wait(lk)
    assert np.array_equal(out, ref)
    for i in range(3):
        assert np.array_equal(lk.phase_time(i)[0], pt[i])
    lk.commit(np.ones(3, np.int32))
    # a second batch through the same worker thread
    lk.submit(nc[:2], pts[:2], par[:2], locs[:2], n0[:2], n1[:2])
    assert np.array_equal(wait(lk), ref[:2])
    # destroyed with a batch in flight: the worker finishes it first
    lk.submit(nc, pts, par, locs, n0, n1)
    lk.close()


def test_one_thread_keeps_tt2d_and_body_contexts_busy(gpulib):
    g2, s2, d2, nc2, pts2, par2, n02, n12 = tt2d_case(63)
    gb, sb, db, ncb, ptsb, parb, locs, n0b, n1b = body_case(64)
    t = TravelTime2DLikelihood(g2, s2, d2, nslots=4, ncell_max=40)
    b = BodyLikelihood(gb, sb, db, nslots=3, ncell_max=30)
    rt = t.forward(nc2, pts2, par2, n02, n12)
    rb = b.forward(ncb, ptsb, parb, locs, n0b, n1b)
    b.submit(ncb, ptsb, parb, locs, n0b, n1b)
    t.submit(nc2, pts2, par2, n02, n12)
    assert np.array_equal(wait(t), rt)
    assert np.array_equal(wait(b), rb)
    t.close(); b.close()
