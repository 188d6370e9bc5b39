"""GPU parity: nearest-nucleus gridding vs the kdtree2 oracle, bit-exact."""
import ctypes

import numpy as np
import pytest

from mctomo_gb300 import kdtree_to_grid, synthetic

pytestmark = pytest.mark.gpu
P = lambda a: None if a is None else a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731


def oracle_grid(orc, pts, par, nx, ny, nz, lo, st, box=None):
    d = pts.shape[1]
    shape = (nx, ny, nz) if d == 3 else (nx, ny)
    sid = np.zeros(shape, np.int32)
    vp = np.zeros(shape); vs = np.zeros(shape); rho = np.zeros(shape)
    b = box if box is not None else [1, nx, 1, ny, 1, nz if d == 3 else 1]
    rc = orc.orc_kdtree_to_grid(d, pts.shape[0], P(np.ascontiguousarray(pts)), P(np.ascontiguousarray(par)),
                                nx, ny, nz if d == 3 else 1, lo[0], lo[1], lo[2] if d == 3 else 0.0,
                                st[0], st[1], st[2] if d == 3 else 0.0, *b, P(sid), P(vp), P(vs), P(rho))
    assert rc == 0
    return sid, vp, vs, rho


@pytest.mark.parametrize("shape,ncell,seed", [((41, 41, 31), 400, 1), ((51, 40, 21), 800, 2),
                                              ((20, 17, 9), 4, 3), ((33, 29, 25), 1500, 4)])
def test_grid_3d_matches_oracle(orc, gpulib, shape, ncell, seed):
    rng = np.random.default_rng(seed)
    nx, ny, nz = shape
    lo = np.array([-3.0, 1.0, 0.0]); st = np.array([1.0, 0.9, 0.2])
    hi = lo + st * (np.array(shape) - 1)
    pts, par = synthetic.voronoi_model_3d(rng, ncell, lo, hi, (0.3, 2.5))
    got = kdtree_to_grid(pts, par, nx, ny, nz, lo, st)
    exp = oracle_grid(orc, pts, par, nx, ny, nz, lo, st)
    for g, e in zip(got, exp):
        np.testing.assert_array_equal(g, e)


def test_grid_2d_matches_oracle(orc, gpulib):
    rng = np.random.default_rng(11)
    nx = ny = 51
    lo = np.array([0.0, 0.0]); st = np.array([0.2, 0.2])
    for n in (4, 20, 100):
        pts = rng.uniform(0, 10, (n, 2))
        par = np.stack([rng.uniform(2, 4, n), rng.uniform(1, 2, n), rng.uniform(2, 3, n)], 1)
        got = kdtree_to_grid(pts, par, nx, ny, 1, lo, st)
        exp = oracle_grid(orc, pts, par, nx, ny, 1, lo, st)
        for g, e in zip(got, exp):
            np.testing.assert_array_equal(g, e)


def test_grid_box_recompute_keeps_outside(orc, gpulib):
    rng = np.random.default_rng(5)
    nx, ny, nz = 30, 25, 12
    lo = np.zeros(3); st = np.array([0.5, 0.5, 0.25])
    pts, par = synthetic.voronoi_model_3d(rng, 120, lo, lo + st * (np.array([nx, ny, nz]) - 1), (0.5, 2.0))
    base = kdtree_to_grid(pts, par, nx, ny, nz, lo, st)
    pts2 = pts.copy(); pts2[7] += 0.3
    box = [5, 17, 3, 20, 2, 11]
    got = kdtree_to_grid(pts2, par, nx, ny, nz, lo, st, box=box,
                         sites_id=base[0].copy(), vp=base[1].copy(), vs=base[2].copy(), rho=base[3].copy())
    exp = [a.copy() for a in base]
    e2 = oracle_grid(orc, pts2, par, nx, ny, nz, lo, st, box=box)
    sl = (slice(4, 17), slice(2, 20), slice(1, 11))
    for a, b in zip(exp, e2):
        a[sl] = b[sl]
    for g, e in zip(got, exp):
        np.testing.assert_array_equal(g, e)


def test_grid_exact_ties_follow_kdtree_rule(orc, gpulib):
    # nuclei mirrored across grid planes: many nodes are exactly equidistant
    # from two or more nuclei, so the kd-tree visiting order decides
    nx, ny, nz = 21, 21, 11
    lo = np.zeros(3); st = np.array([1.0, 1.0, 1.0])
    rng = np.random.default_rng(9)
    base = rng.integers(1, 19, (60, 3)).astype(float)
    base[:, 2] = rng.integers(1, 10, 60)
    pts = np.concatenate([base + [0.5, 0, 0], base - [0.5, 0, 0], base + [0, 0.5, 0.5]])
    pts = np.unique(pts, axis=0)
    par = np.stack([np.arange(len(pts)) + 1.0, np.arange(len(pts)) * 0.5 + 1, np.ones(len(pts))], 1)
    got = kdtree_to_grid(pts, par, nx, ny, nz, lo, st)
    exp = oracle_grid(orc, pts, par, nx, ny, nz, lo, st)
    np.testing.assert_array_equal(got[0], exp[0])
    np.testing.assert_array_equal(got[1], exp[1])


def test_grid_deterministic_repeat(gpulib):
    rng = np.random.default_rng(12)
    lo = np.zeros(3); st = np.array([0.5, 0.5, 0.5])
    pts, par = synthetic.voronoi_model_3d(rng, 300, lo, lo + st * 40, (0.3, 2.5))
    a = kdtree_to_grid(pts, par, 41, 41, 41, lo, st)
    b = kdtree_to_grid(pts, par, 41, 41, 41, lo, st)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)


@pytest.mark.parametrize("k,shape,lo,st", [
    (1, (41, 51, 31), (-2.0, -2.0, 0.0), (0.1, 0.1, 0.1)),
    (2, (51, 141, 21), (0.0, 0.0, 0.0), (0.1, 0.1, 0.1)),
])
def test_grid_reference_vertices_match_oracle(orc, gpulib, k, shape, lo, st):
    # the Voronoi nuclei the reference ships (plot/run_time_vertices_k.txt,
    # fixture made by tests/golden/make_vertices.py), gridded at 0.1 km
    import os
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "reference_vertices.npz"))
    pts, val = d["pts%d" % k], d["val%d" % k]
    par = np.ascontiguousarray(np.column_stack([val[:, 0], val[:, 1], np.full(len(pts), 2.0)]))
    lo = np.array(lo); st = np.array(st)
    nx, ny, nz = shape
    got = kdtree_to_grid(np.ascontiguousarray(pts), par, nx, ny, nz, lo, st)
    exp = oracle_grid(orc, np.ascontiguousarray(pts), par, nx, ny, nz, lo, st)
    for g, e in zip(got, exp):
        np.testing.assert_array_equal(g, e)
