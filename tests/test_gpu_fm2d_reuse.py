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
