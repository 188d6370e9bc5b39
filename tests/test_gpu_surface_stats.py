"""GPU: posterior statistics of the committed models on the device
(mct_surf_stat_*, the reference's stat_rti and write_mean / write_var)
against the same sums taken on the host over the oracle's gridding of the
committed models, bit for bit; slots are counted separately and reset."""
import ctypes

import numpy as np
import pytest

from mctomo_gb300 import SurfaceLikelihood, synthetic
from test_gpu_surface import small_case

pytestmark = pytest.mark.gpu
P = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731


def grids(orc, grid, n, pts, par):
    shape = (grid["nx"], grid["ny"], grid["nz"])
    sid = np.zeros(shape, np.int32)
    vp, vs, rho = np.zeros(shape), np.zeros(shape), np.zeros(shape)
    orc.orc_kdtree_to_grid(3, int(n), P(np.ascontiguousarray(pts[:n])), P(np.ascontiguousarray(par[:n])), *shape,
                           grid["xmin"], grid["ymin"], grid["zmin"], grid["dx"], grid["dy"], grid["dz"], 1, shape[0],
                           1, shape[1], 1, shape[2], P(sid), P(vp), P(vs), P(rho))
    return vp, vs


def test_posterior_sums_of_committed_models(orc, gpulib):
    rng, grid, settings, data, ncells, pts, par = small_case(71, nchains=4, ncell_max=60)
    settings["material_law"] = 0        # vp, vs from the nucleus parameters
    par[:, :, 0] = par[:, :, 1] * 1.73
    npd = len(data["freqs"])
    lk = SurfaceLikelihood(grid, settings, data, nslots=4, ncell_max=60)
    slots = np.arange(4, dtype=np.int32)
    n0, n1 = np.full((4, npd), 0.02), np.zeros((4, npd))
    lk.forward(slots, ncells, pts, par, n0, n1)
    lk.commit(np.ones(4, np.int32))
    cur = [(pts[c].copy(), par[c].copy()) for c in range(4)]
    acc = {c: [np.zeros((grid["nx"], grid["ny"], grid["nz"])) for _ in range(4)] for c in range(4)}
    count = [0] * 4

    def add(cs):
        lk.stat_add(cs)
        for c in cs:
            vp, vs = grids(orc, grid, ncells[c], *cur[c])
            a = acc[c]
            a[0] = a[0] + vp; a[1] = a[1] + vs; a[2] = a[2] + vp * vp; a[3] = a[3] + vs * vs
            count[c] += 1

    add([0, 2])
    p, q = pts, par
    for step in range(3):
        p, q = synthetic.perturb_chain_models(rng, ncells, p, q, grid)
        q = q.copy(); q[:, :, 0] = q[:, :, 1] * 1.73
        lk.forward(slots, ncells, p, q, n0, n1)
        accept = np.array([1, 0, 1, step % 2], np.int32)
        lk.commit(accept)
        for c in range(4):
            if accept[c]:
                cur[c] = (p[c].copy(), q[c].copy())
        add([0, 1, 2, 3] if step != 1 else [3, 1])
    for c in range(4):
        mp, ms, qp, qs, n = lk.stat_read(c)
        assert n == count[c]
        for got, s in zip((mp, ms, qp, qs), acc[c]):
            np.testing.assert_array_equal(got, s / n)
    lk.stat_reset(1)
    mp, ms, qp, qs, n = lk.stat_read(1)
    assert n == 0 and not mp.any() and not qs.any()
    # a slot claimed afresh (mct_surf_admit: slot 0, the first free one)
    # starts with no statistics
    assert lk.stat_read(0)[4] == count[0] > 0
    assert lk.admit() == 0
    assert lk.stat_read(0)[4] == 0
    assert lk.stat_read(2)[4] == count[2]
    lk.close()
