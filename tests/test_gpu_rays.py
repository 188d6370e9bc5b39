"""GPU parity of ray-path group delays (modrays with uar = 0, i.e. rpaths,
then CalGroupTime) against the oracle's restatement: bit-for-bit with FP64
travel times (precision 0), within the travel-time bound with double-float
times (precision 1)."""
import ctypes

import numpy as np
import pytest

from mctomo_gb300 import modrays_group_batch, synthetic

pytestmark = pytest.mark.gpu
P = lambda a: None if a is None else a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
TT_TOL = 1e-4


def oracle_group(orc, st, srs, nv, h, velv, gvel, asgr, sgdl, sgs, fom):
    n = len(st)
    sx, sz = np.ascontiguousarray(st[:, 0]), np.ascontiguousarray(st[:, 1])
    tt = np.zeros((n, n)); gt = np.zeros((n, n)); ln = np.zeros((n, n)); cz = ctypes.c_int()
    rc = orc.orc_modrays_group(n, P(sx), P(sz), n, P(sx), P(sz), P(np.ascontiguousarray(srs, np.int32)), nv, nv,
                               0.0, 0.0, h, h, P(np.ascontiguousarray(velv)), 1, 1, asgr, sgdl, sgs, fom,
                               P(np.ascontiguousarray(gvel)), P(tt), P(gt), P(ln), ctypes.byref(cz))
    assert rc == 0
    return tt, gt, ln, cz.value


@pytest.mark.parametrize("asgr,fom", [(1, 1), (1, 0), (0, 1)])
def test_group_delays_match_oracle(orc, gpulib, asgr, fom):
    rng = np.random.default_rng(60 + asgr * 2 + fom)
    nv, h, nmaps = 41, 1.0, 3
    velv = synthetic.voronoi_phase_maps(rng, nmaps, nv, nv, h, h, ncell=30, vrange=(0.6, 2.0))
    gvel = velv[:, 1:-1, 1:-1] * 0.8
    st = rng.uniform(3.0, 37.0, (10, 2))
    srs = np.triu(np.ones((10, 10), np.int32), 1)
    m = srs == 1
    # without source refinement rays can circle the source cell (the
    # reference takes the gradient at the cell's lower-left node) and the
    # circling is chaotic: only the exact FP64 path is compared there
    for prec, tol in ((0, 1e-9), (1, TT_TOL)) if asgr == 1 else ((0, 1e-9),):
        tt, gt, ln, cz = modrays_group_batch(st, st, srs, nv, nv, 0.0, 0.0, h, h, velv, gvel, asgr=asgr, fom=fom,
                                             precision=prec)
        for mp in range(nmaps):
            ett, egt, eln, ecz = oracle_group(orc, st, srs, nv, h, velv[mp], gvel[mp], asgr, 4, 8, fom)
            assert cz[mp] == ecz
            assert np.max(np.abs(tt[mp][m] - ett[m])) <= tol
            assert np.max(np.abs(gt[mp][m] - egt[m])) <= tol, (prec, np.max(np.abs(gt[mp][m] - egt[m])))
            assert np.max(np.abs(ln[mp][m] - eln[m])) <= tol * 2


def test_group_delays_homogeneous(gpulib):
    nv, h = 41, 0.5
    st = np.array([[3.1, 4.2], [17.3, 5.6], [9.9, 16.4], [15.2, 15.9]])
    srs = 1 - np.eye(4, dtype=np.int32)
    velv = np.full((1, nv + 2, nv + 2), 2.0)
    gvel = np.full((1, nv, nv), 1.6)
    tt, gt, ln, cz = modrays_group_batch(st, st, srs, nv, nv, 0.0, 0.0, h, h, velv, gvel)
    m = srs == 1
    d = np.hypot(st[:, None, 0] - st[None, :, 0], st[:, None, 1] - st[None, :, 1])
    assert cz[0] == 0
    np.testing.assert_allclose(gt[0][m], ln[0][m] / 1.6, rtol=1e-12)
    assert np.all(ln[0][m] >= d[m] * (1 - 1e-9)) and np.all(ln[0][m] <= d[m] * 1.02)
