"""GPU: a context's SM share (mct_surf_set_sm_share, mct_tt2d_set_sm_share)
changes only how many blocks the fm2d solve kernels launch; every block then
walks several logical blocks in turn. Times and -log L stay the same bits as
with the whole device, and out-of-range shares are refused."""
import numpy as np
import pytest

from mctomo_gb300 import MctError, SurfaceLikelihood, TravelTime2DLikelihood, synthetic

pytestmark = pytest.mark.gpu

# 0.004 x 152 SMs rounds to one SM: the solve kernels get one SM's worth of
# blocks, far fewer than their logical blocks
TINY = 0.004


def test_tt2d_share_gives_the_same_times(gpulib):
    rng = np.random.default_rng(31)
    g, s, d = synthetic.tt2d_workload(rng, nx=41, ny=41, nstations=12)
    nch = 6
    nc, pts, par = synthetic.tt2d_chain_models(rng, nch, 40, g, (4, 40))
    n0, n1 = np.zeros((nch, 2)), np.full((nch, 2), 0.05)
    lk = TravelTime2DLikelihood(g, s, d, nslots=nch, ncell_max=40)
    full = lk.forward(nc, pts, par, n0, n1)
    tf = [lk.phase_time(i) for i in range(nch)]
    for share in (TINY, 0.3, 1.0, 0.0):
        lk.set_sm_share(share)
        out = lk.forward(nc, pts, par, n0, n1)
        assert np.array_equal(out, full), share
        for i in range(nch):
            assert np.array_equal(lk.phase_time(i), tf[i]), (share, i)
    for bad in (-0.1, 1.5, float("nan")):
        with pytest.raises(MctError):
            lk.set_sm_share(bad)


def test_surface_share_gives_the_same_times(gpulib):
    rng = np.random.default_rng(32)
    g, s, d = synthetic.surface_workload(rng, nx=21, ny=19, nz=11, extent=(20.0, 18.0, 3.0), nstations=10,
                                         nperiods=4, pmin=0.5, pmax=3.0)
    nch = 4
    nc, pts, par = synthetic.surface_chain_models(rng, nch, 40, g, (6, 40))
    slots = np.arange(nch, dtype=np.int32)
    n0, n1 = np.full((nch, 4), 0.02), np.zeros((nch, 4))
    lk = SurfaceLikelihood(g, s, d, nslots=nch, ncell_max=40)
    full = lk.forward(slots, nc, pts, par, n0, n1)
    tf = [lk.phase_time(i)[0] for i in range(nch)]
    lk.set_sm_share(TINY)
    out = lk.forward(slots, nc, pts, par, n0, n1)
    assert np.array_equal(out, full)
    for i in range(nch):
        assert np.array_equal(lk.phase_time(i)[0], tf[i]), i
    # the asynchronous path launches with the same share
    lk.submit(slots, nc, pts, par, n0, n1)
    done, got = lk.poll()
    while not done:
        done, got = lk.poll()
    assert np.array_equal(got, full)
