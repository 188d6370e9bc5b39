"""Serving API of the surface context: device-memory sizing (host logic,
runs without a GPU), asynchronous submit/poll against the blocking forward,
and the chain-slot allocator."""
import time

import numpy as np
import pytest

from mctomo_gb300 import MctError, SurfaceLikelihood, synthetic
from mctomo_gb300.surface import device_bytes


def small(seed, nslots=4, ncell_max=30):
    rng = np.random.default_rng(seed)
    grid, settings, data = synthetic.surface_workload(rng, nx=21, ny=19, nz=11, extent=(20.0, 18.0, 3.0),
                                                      nstations=8, nperiods=4, pmin=0.5, pmax=3.0)
    ncells, pts, par = synthetic.surface_chain_models(rng, nslots, ncell_max, grid, ncell_range=(6, ncell_max))
    return rng, grid, settings, data, ncells, pts, par


def test_device_bytes_grows_with_slots(gpulib):
    _, grid, settings, data, *_ = small(1)
    b1 = device_bytes(grid, settings, data, 1, 30)
    b4 = device_bytes(grid, settings, data, 4, 30)
    b8 = device_bytes(grid, settings, data, 8, 30)
    assert 0 < b1 < b4 < b8
    # per-slot cost is constant: the context is a fixed part plus slots
    assert abs((b8 - b4) - (b4 - b1) * 4 / 3) < 0.01 * (b8 - b4) + 4096
    with pytest.raises(MctError):
        device_bytes(grid, settings, data, 0, 30)


@pytest.mark.gpu
def test_submit_poll_matches_forward(gpulib):
    rng, grid, settings, data, ncells, pts, par = small(2)
    npd = len(data["freqs"])
    n0 = np.full((4, npd), 0.02); n1 = np.full((4, npd), 0.01)
    slots = np.arange(4)
    a = SurfaceLikelihood(grid, settings, data, nslots=4, ncell_max=pts.shape[1])
    b = SurfaceLikelihood(grid, settings, data, nslots=4, ncell_max=pts.shape[1])
    ref = a.forward(slots, ncells, pts, par, n0, n1)
    b.submit(slots, ncells, pts, par, n0, n1)
    # blocking calls are refused while a batch is in flight
    with pytest.raises(MctError):
        b.forward(slots, ncells, pts, par, n0, n1)
    t0 = time.time()
    done, out = b.poll()
    while not done:
        assert time.time() - t0 < 60
        time.sleep(0.001)
        done, out = b.poll()
    np.testing.assert_array_equal(out, ref)
    with pytest.raises(MctError):
        b.poll()               # nothing pending
    b.commit(np.ones(4, np.int32))
    a.commit(np.ones(4, np.int32))
    pts2, par2 = synthetic.perturb_chain_models(rng, ncells, pts, par, grid)
    b.submit(slots, ncells, pts2, par2, n0, n1)
    ref2 = a.forward(slots, ncells, pts2, par2, n0, n1)
    done = False
    while not done:
        done, out2 = b.poll()
    np.testing.assert_array_equal(out2, ref2)
    a.close(); b.close()


@pytest.mark.gpu
def test_admit_evict_slots(gpulib):
    rng, grid, settings, data, ncells, pts, par = small(3, nslots=3)
    npd = len(data["freqs"])
    n0 = np.full((1, npd), 0.02); n1 = np.full((1, npd), 0.01)
    lk = SurfaceLikelihood(grid, settings, data, nslots=3, ncell_max=pts.shape[1])
    got = [lk.admit() for _ in range(3)]
    assert sorted(got) == [0, 1, 2]
    with pytest.raises(MctError):
        lk.admit()
    # chain in slot 1 commits a model, then leaves; a new chain admitted into
    # the slot starts from nothing committed (all columns recomputed), which
    # gives the same result as a fresh context
    lk.forward(np.array([1]), ncells[:1], pts[:1], par[:1], n0, n1)
    lk.commit(np.ones(1, np.int32))
    lk.evict(1)
    with pytest.raises(MctError):
        lk.evict(1)
    assert lk.admit() == 1
    out = lk.forward(np.array([1]), ncells[2:3], pts[2:3], par[2:3], n0, n1)
    fresh = SurfaceLikelihood(grid, settings, data, nslots=1, ncell_max=pts.shape[1])
    exp = fresh.forward(np.array([0]), ncells[2:3], pts[2:3], par[2:3], n0, n1)
    np.testing.assert_array_equal(out, exp)
    fresh.close(); lk.close()
