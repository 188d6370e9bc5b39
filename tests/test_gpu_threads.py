"""GPU: the per-solve drop-in calls from several host threads at once.

The reference calls fastMarching3D from an OpenMP loop over stations
(src/likelihood_body.F90:204-224) and modrays per period from an OpenMP loop
(src/likelihood_surf.F90:295-334). Each host thread has its own stream and
workspace in the library, so concurrent calls must give the same results as
the same calls made one after another (bit for bit), and the oracle's.
"""
import concurrent.futures as cf
import ctypes

import numpy as np
import pytest

from mctomo_gb300 import fast_marching3d, modrays

pytestmark = pytest.mark.gpu
P = lambda a: None if a is None else a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731


def _eik3_cases(n):
    rng = np.random.default_rng(31)
    shape = (23, 19, 13)
    vels = [3.0 + rng.random(shape) for _ in range(n)]
    srcs = [rng.uniform([1, 1, 0.5], [20, 16, 5.5]) for _ in range(n)]
    rev = rng.uniform([1, 1, 0], [20, 16, 5], (17, 3))
    return shape, vels, srcs, rev


@pytest.mark.parametrize("order", [0, 1])
def test_fast_marching3d_from_threads_matches_serial(orc, gpulib, order):
    shape, vels, srcs, rev = _eik3_cases(24)
    h, lo = (1.0, 1.0, 0.5), (0.0, 0.0, 0.0)

    def one(i):
        return fast_marching3d(vels[i], h, lo, srcs[i], rev, order=order)

    serial = [one(i) for i in range(len(vels))]
    with cf.ThreadPoolExecutor(8) as ex:
        threaded = list(ex.map(one, range(len(vels))))
    for a, b in zip(serial, threaded):
        np.testing.assert_array_equal(a, b)
    # and the reference's own solver (oracle restatement, pinned to it)
    tol = 1e-4 if order == 0 else 0.0
    for i in (0, 7, 23):
        et = np.zeros(len(rev))
        orc.orc_fast_marching3d(*shape, *h, *lo, P(np.ascontiguousarray(vels[i])), P(np.ascontiguousarray(srcs[i])),
                                P(np.ascontiguousarray(rev)), len(rev), order, P(et), None)
        assert np.max(np.abs(threaded[i] - et)) <= tol


def test_modrays_from_threads_matches_serial(gpulib):
    rng = np.random.default_rng(32)
    nv = 21
    sta = rng.uniform(3.0, 17.0, (6, 2))
    srs = np.triu(np.ones((6, 6), np.int32), 1)
    maps = [1.0 + rng.random((nv + 2, nv + 2)) for _ in range(16)]

    def one(i):
        return modrays(sta, sta, srs, nv, nv, 0.0, 0.0, 1.0, 1.0, maps[i], sgdl=4, sgs=4)

    serial = [one(i) for i in range(len(maps))]
    with cf.ThreadPoolExecutor(8) as ex:
        threaded = list(ex.map(one, range(len(maps))))
    for a, b in zip(serial, threaded):
        np.testing.assert_array_equal(a, b)
