"""GPU: the surface context reuses a committed refined source box when the
proposal's phase map is unchanged over the box and the B-spline's reach;
the travel times and -log L are the same bits as a context evaluating the
proposal with nothing committed (every box marched), over several
accept / reject steps."""
import numpy as np
import pytest

from mctomo_gb300 import SurfaceLikelihood, synthetic
from test_gpu_surface import small_case

pytestmark = pytest.mark.gpu


def test_reused_boxes_give_the_marched_results(gpulib):
    rng, grid, settings, data, ncells, pts, par = small_case(91, nchains=4, ncell_max=60)
    npd = len(data["freqs"])
    slots = np.arange(4, dtype=np.int32)
    n0, n1 = np.full((4, npd), 0.02), np.zeros((4, npd))
    lk = SurfaceLikelihood(grid, settings, data, nslots=4, ncell_max=60)
    lk.forward(slots, ncells, pts, par, n0, n1)
    lk.commit(np.ones(4, np.int32))
    p, q = pts, par
    for step in range(4):
        p2, q2 = synthetic.perturb_chain_models(rng, ncells, p, q, grid)
        got = lk.forward(slots, ncells, p2, q2, n0, n1)
        pt = [lk.phase_time(c)[0] for c in range(4)]
        fresh = SurfaceLikelihood(grid, settings, data, nslots=4, ncell_max=60)
        exp = fresh.forward(slots, ncells, p2, q2, n0, n1)
        for c in range(4):
            np.testing.assert_array_equal(pt[c], fresh.phase_time(c)[0])
        np.testing.assert_array_equal(got, exp)
        fresh.close()
        accept = np.array([1, step % 2, 0, 1], np.int32)
        lk.commit(accept)
        for c in range(4):
            if accept[c]:
                p = p.copy(); q = q.copy()
                p[c], q[c] = p2[c], q2[c]
    lk.close()


def test_reused_boxes_in_the_2d_context(gpulib):
    from mctomo_gb300 import TravelTime2DLikelihood
    rng = np.random.default_rng(92)
    grid, settings, data = synthetic.tt2d_workload(rng)
    nch = 6
    ncells, pts, par = synthetic.tt2d_chain_models(rng, nch, 100, grid)
    n0, n1 = np.zeros((nch, 2)), np.full((nch, 2), 0.05)
    lk = TravelTime2DLikelihood(grid, settings, data, nslots=nch, ncell_max=100)
    lk.forward(ncells, pts, par, n0, n1)
    lk.commit(np.ones(nch, np.int32))
    p, q = pts, par
    for step in range(4):
        # a value change of one cell per chain (the 2D sampler's commonest step)
        q2 = q.copy()
        for c in range(nch):
            i = rng.integers(ncells[c])
            q2[c, i, 0] = rng.uniform(2.0, 4.0)
        got = lk.forward(ncells, p, q2, n0, n1)
        fresh = TravelTime2DLikelihood(grid, settings, data, nslots=nch, ncell_max=100)
        exp = fresh.forward(ncells, p, q2, n0, n1)
        for c in range(nch):
            np.testing.assert_array_equal(lk.phase_time(c), fresh.phase_time(c))
        np.testing.assert_array_equal(got, exp)
        fresh.close()
        accept = (rng.random(nch) < 0.5).astype(np.int32)
        lk.commit(accept)
        q = np.where(accept[:, None, None] == 1, q2, q)
    lk.close()
