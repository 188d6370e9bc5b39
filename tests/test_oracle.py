"""CPU tests of the oracle (the checker) against the reference's golden
vectors and against analytic known answers."""
import ctypes
import os

import numpy as np
import pytest

import oracle

GOLD = os.path.join(os.path.dirname(__file__), "golden", "fmm3d_ref.npz")
P = lambda a: None if a is None else a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731


def test_sfmm3d_oracle_matches_reference_golden(orc):
    g = np.load(GOLD)
    for i in range(int(g["ncases"])):
        c = {k[len("c%d_" % i):]: g[k] for k in g.files if k.startswith("c%d_" % i)}
        vel = np.ascontiguousarray(c["vel"])
        rev = np.ascontiguousarray(c["rev"])
        tt = np.zeros(rev.shape[0])
        tf = np.zeros_like(vel)
        rc = orc.orc_fast_marching3d(int(c["nx"]), int(c["ny"]), int(c["nz"]), *c["h"], *c["lo"],
                                     P(vel), P(np.ascontiguousarray(c["src"])), P(rev), rev.shape[0],
                                     int(c["order"]), P(tt), P(tf))
        assert rc == 0
        np.testing.assert_array_equal(tf, c["tfield"])
        np.testing.assert_array_equal(tt, c["ttime"])


def test_sfmm3d_oracle_matches_compiled_reference(orc):
    ref = oracle.load_reference()
    if ref is None:
        pytest.skip("reference fastMarching3D not built on this host")
    rng = np.random.default_rng(7)
    for trial in range(4):
        nx, ny, nz = (int(v) for v in rng.integers(8, 24, 3))
        vel = rng.uniform(3.0, 7.5, (nx, ny, nz))
        src = np.array([rng.uniform(0.5, nx - 1.5), rng.uniform(0.5, ny - 1.5), rng.uniform(0.5, nz - 1.5)]) * 0.5
        rev = np.stack([rng.uniform(0, nx - 1.2, 9), rng.uniform(0, ny - 1.2, 9), rng.uniform(0, nz - 1.2, 9)], 1) * 0.5
        for order in (0, 1):
            a = [np.zeros(9), np.zeros((nx, ny, nz))]
            b = [np.zeros(9), np.zeros((nx, ny, nz))]
            orc.orc_fast_marching3d(nx, ny, nz, .5, .5, .5, 0., 0., 0., P(vel), P(src), P(rev), 9, order, P(a[0]), P(a[1]))
            ref.fastMarching3D(nx, ny, nz, .5, .5, .5, 0., 0., 0., P(vel), P(src), P(rev), 9, order, P(b[0]), P(b[1]))
            np.testing.assert_array_equal(a[1], b[1])
            np.testing.assert_array_equal(a[0], b[0])


def test_kdtree_oracle_equals_brute_force(orc):
    rng = np.random.default_rng(3)
    for d in (2, 3):
        pts = np.ascontiguousarray(rng.uniform(-5, 5, (257, d)))
        for _ in range(500):
            q = rng.uniform(-6, 6, d)
            i = orc.orc_kdtree_nearest(d, pts.shape[0], P(pts), P(q))
            assert i == np.argmin(((pts - q) ** 2).sum(1)) + 1


def test_kdtree_oracle_tie_rule_is_a_minimiser(orc):
    # nuclei mirrored about grid nodes: every tie must resolve to one of the
    # equidistant nuclei, deterministically
    pts = np.array([[0.5, 0.0, 0.0], [-0.5, 0.0, 0.0], [0.0, 0.5, 0.0], [0.0, -0.5, 0.0],
                    [2.0, 2.0, 2.0], [3.0, 3.0, 1.0]] * 3, float)
    pts = np.ascontiguousarray(pts + np.repeat(np.arange(3), 6)[:, None] * 4.0)
    q = np.array([0.0, 0.0, 0.0])
    i = orc.orc_kdtree_nearest(3, pts.shape[0], P(pts), P(q))
    d = ((pts - q) ** 2).sum(1)
    assert d[i - 1] == d.min()
    assert orc.orc_kdtree_nearest(3, pts.shape[0], P(pts), P(q)) == i


def test_surfdisp_rayleigh_halfspace_known_answer(orc):
    # Poisson solid half-space: c_R / beta = 0.919402 (root of the Rayleigh equation)
    vs = np.array([1.5, 1.5], np.float32)
    vp = (vs * np.float32(np.sqrt(3.0))).astype(np.float32)
    rho = np.array([2.0, 2.0], np.float32)
    th = np.array([2.0, 0.0], np.float32)
    per = np.array([0.5, 1.0, 3.0, 10.0])
    cp = np.zeros(4); cg = np.zeros(4)
    ierr = orc.orc_surfdisp96(P(th), P(vp), P(vs), P(rho), 2, 2, 1, 0, 4, P(per), 0.001, P(cp), P(cg), None)
    assert ierr == 0
    x = np.linspace(0.85, 0.95, 200001)
    f = (2 - x ** 2) ** 2 - 4 * np.sqrt(1 - x ** 2 / 3) * np.sqrt(1 - x ** 2)
    root = x[np.argmin(np.abs(f))] * 1.5
    np.testing.assert_allclose(cp, root, atol=2e-5)


def test_surfdisp_love_layer_over_halfspace_known_answer(orc):
    from scipy.optimize import brentq
    b1, b2, r1, r2, h = 1.0, 2.0, 2.0, 2.5, 1.0
    vs = np.array([b1, b2], np.float32)
    vp = (vs * np.float32(1.73)).astype(np.float32)
    rho = np.array([r1, r2], np.float32)
    th = np.array([h, 0.0], np.float32)
    per = np.linspace(0.5, 5.0, 10)
    cp = np.zeros(10); cg = np.zeros(10)
    ierr = orc.orc_surfdisp96(P(th), P(vp), P(vs), P(rho), 2, 1, 1, 0, 10, P(per), 0.001, P(cp), P(cg), None)
    assert ierr == 0

    def f(c, T):
        k = 2 * np.pi / T / c
        s1 = np.sqrt(c * c / b1 ** 2 - 1)
        s2 = np.sqrt(1 - c * c / b2 ** 2)
        return np.sin(k * h * s1) * r1 * b1 ** 2 * s1 - np.cos(k * h * s1) * r2 * b2 ** 2 * s2

    for c, T in zip(cp, per):
        # fundamental branch: k h s1 in (0, pi/2)
        cmax = min(b2 * (1 - 1e-12), b1 * np.sqrt(1 + (np.pi / 2 / (2 * np.pi / T / b2 * h)) ** 2))
        lo = b1 * (1 + 1e-9)
        hi = cmax
        while f(hi, T) * f(lo, T) > 0 and hi > lo:
            hi = lo + (hi - lo) * 0.999
        root = brentq(f, lo, min(hi, b2 * (1 - 1e-12)), args=(T,), xtol=1e-12)
        assert abs(c - root) < 2e-5, (T, c, root)


def test_fm2d_homogeneous_converges_to_straight_line_time(orc):
    nvx = nvz = 41
    v = 3.0
    velv = np.asfortranarray(np.full((nvz + 2, nvx + 2), v))
    sx, sz = np.array([3.3]), np.array([4.1])
    rx, rz = np.array([8.7, 1.1, 9.6]), np.array([1.2, 9.3, 9.6])
    srs = np.ones(3, np.int32)
    tt = np.zeros(3)
    rc = orc.orc_modrays(1, P(sx), P(sz), 3, P(rx), P(rz), P(srs), nvx, nvz, 0., 0., 0.25, 0.25,
                         P(velv), 1, 1, 1, 4, 8, 1, 0.5, P(tt), None)
    assert rc == 0
    exact = np.hypot(rx - sx, rz - sz) / v
    assert np.all(np.abs(tt - exact) / exact < 0.01)


def test_misfit_reduction_hand_computed(orc):
    nsrc, nrev, np_ = 2, 2, 1
    phase = np.array([1.0, 2.0, 3.0, 4.0])      # (nrev, nsrc, np)
    obs = np.zeros((np_, 3, 4))
    obs[0, 0] = [1.1, 2.0, 2.5, 4.0]
    obs[0, 1] = 0.1
    raystat = np.zeros((np_, 2, 4), np.int32)
    raystat[0, 0] = [1, 1, 0, 1]
    sig = np.zeros(4); out = np.zeros(3)
    n0 = np.array([0.0]); n1 = np.array([0.1])
    rc = orc.orc_surf_misfit(nsrc, nrev, np_, P(phase), P(np.ascontiguousarray(obs)), P(np.ascontiguousarray(raystat)),
                             P(phase), 1, P(n0), P(n1), 3, P(sig), P(out))
    assert rc == 0
    r = np.array([-0.1, 0.0, 0.0])
    s = 0.1
    like = (r ** 2 / (2 * s * s)).sum() + 3 * np.log(0.1) + np.log(1.0) + 1.5 * np.log(np.float64(np.float32(6.283185)))
    np.testing.assert_allclose(out, [like, (r ** 2 / s ** 2).sum(), (r ** 2).sum()], rtol=1e-12)


def _modrays_group(orc, st, srs, nv, h, velv, gvel, asgr=1, sgdl=4, sgs=8, fom=1):
    n = len(st)
    sx, sz = np.ascontiguousarray(st[:, 0]), np.ascontiguousarray(st[:, 1])
    tt = np.zeros((n, n)); gt = np.zeros((n, n)); ln = np.zeros((n, n)); cz = ctypes.c_int()
    rc = orc.orc_modrays_group(n, P(sx), P(sz), n, P(sx), P(sz), P(np.ascontiguousarray(srs, np.int32)), nv, nv,
                               0.0, 0.0, h, h, P(np.ascontiguousarray(velv)), 1, 1, asgr, sgdl, sgs, fom,
                               P(np.ascontiguousarray(gvel)), P(tt), P(gt), P(ln), ctypes.byref(cz))
    assert rc == 0
    return tt, gt, ln, cz.value


@pytest.mark.parametrize("asgr", [1, 0])
def test_rays_homogeneous_group_time_is_length_over_velocity(orc, asgr):
    # uniform phase velocity: rays are close to straight lines and the group
    # delay along them is exactly their length over the uniform group velocity
    nv, h = 41, 0.5
    st = np.array([[3.1, 4.2], [17.3, 5.6], [9.9, 16.4], [15.2, 15.9]])
    n = len(st)
    srs = 1 - np.eye(n, dtype=np.int32)
    velv = np.full((nv + 2, nv + 2), 2.0)
    gvel = np.full((nv, nv), 1.6)
    tt, gt, ln, cz = _modrays_group(orc, st, srs, nv, h, velv, gvel, asgr=asgr)
    assert cz == 0
    d = np.hypot(st[:, None, 0] - st[None, :, 0], st[:, None, 1] - st[None, :, 1])
    m = srs == 1        # [source][receiver], as ttime
    np.testing.assert_allclose(gt[m], ln[m] / 1.6, rtol=1e-12)
    assert np.all(ln[m] >= d[m] * (1 - 1e-9))
    if asgr == 1:
        assert np.all(ln[m] <= d[m] * 1.02)
    # without refinement the reference takes the gradient at the cell's
    # lower-left node, and rays may circle the source cell before they end
    # FMM discretisation (first order near the source without refinement)
    np.testing.assert_allclose(tt[m], d[m] / 2.0, rtol=0.05 if asgr == 1 else 0.1)


def test_rays_phase_times_unchanged_by_ray_tracing(orc):
    rng = np.random.default_rng(3)
    nv, h = 31, 1.0
    st = rng.uniform(3.0, 27.0, (6, 2))
    srs = np.triu(np.ones((6, 6), np.int32), 1)
    velv = rng.uniform(1.0, 2.0, (nv + 2, nv + 2))
    gvel = rng.uniform(0.8, 1.6, (nv, nv))
    tt, gt, ln, cz = _modrays_group(orc, st, srs, nv, h, velv, gvel)
    tt0 = np.zeros((6, 6))
    sx, sz = np.ascontiguousarray(st[:, 0]), np.ascontiguousarray(st[:, 1])
    assert orc.orc_modrays(6, P(sx), P(sz), 6, P(sx), P(sz), P(srs), nv, nv, 0.0, 0.0, h, h, P(velv), 1, 1, 1, 4, 8,
                           1, 0.5, P(tt0), None) == 0
    m = srs == 1
    np.testing.assert_array_equal(tt[m], tt0[m])
    d = np.hypot(st[:, None, 0] - st[None, :, 0], st[:, None, 1] - st[None, :, 1])
    assert np.all(ln[m] >= d[m] * (1 - 1e-9))
    # group times bracketed by the extreme group velocities along the ray
    assert np.all(gt[m] >= ln[m] / 1.6 * (1 - 1e-12)) and np.all(gt[m] <= ln[m] / 0.8 * (1 + 1e-12))


def test_straight_rays_uniform_velocity(orc):
    nx = ny = 21
    src = np.array([[1.0, 1.5], [8.0, 12.5]])
    rev = np.array([[15.0, 3.0], [2.5, 18.0], [19.0, 19.0]])
    raystat = np.array([1, 1, 0, 1, 0, 1], np.int32)
    vel = np.full((nx, ny), 2.5)
    t = np.zeros(6); d = np.zeros(6)
    rc = orc.orc_straight_group(2, P(np.ascontiguousarray(src)), 3, P(np.ascontiguousarray(rev)), P(raystat), nx, ny,
                                0.0, 0.0, 1.0, 1.0, P(vel), P(t), P(d))
    assert rc == 0
    ds = np.hypot(rev[None, :, 0] - src[:, None, 0], rev[None, :, 1] - src[:, None, 1]).reshape(-1)
    np.testing.assert_allclose(d, ds, rtol=1e-15)
    np.testing.assert_allclose(t[raystat == 1], ds[raystat == 1] / 2.5, rtol=1e-12)
    assert np.all(t[raystat == 0] == 0)


def test_kdtree_oracle_on_the_reference_vertices(orc):
    # the nuclei the reference ships with its plots (fixture from
    # tests/golden/make_vertices.py): the kd-tree search returns a nearest
    # nucleus for grid-like queries, the smallest index among exact ties
    # excepted (those follow the kd-tree visiting order)
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "reference_vertices.npz"))
    rng = np.random.default_rng(4)
    for k in (1, 2):
        pts = np.ascontiguousarray(d["pts%d" % k])
        lo, hi = pts.min(0), pts.max(0)
        for _ in range(300):
            q = np.round(rng.uniform(lo, hi) / 0.1) * 0.1
            i = orc.orc_kdtree_nearest(3, pts.shape[0], P(pts), P(np.ascontiguousarray(q)))
            dd = ((pts - q) ** 2).sum(1)
            assert dd[i - 1] == dd.min()


def test_location_readout_c_matches_the_python_restatement(orc):
    # orc_location_times (C, OpenMP) against oracle.location.interpolate3d
    # (plain Python) on random fields, events inside and on the grid's faces
    from oracle import location as oloc
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    rng = np.random.default_rng(5)
    grid = dict(nx=9, ny=7, nz=6, xmin=1.0, ymin=-2.0, zmin=0.5, dx=0.5, dy=0.75, dz=0.4, scaling=2.0)
    fields = rng.uniform(0, 10, (2, 3, 9, 7, 6))
    ev = np.zeros((11, 4))
    ev[:, 0] = rng.uniform(1.0, 5.0, 11); ev[:, 1] = rng.uniform(-2.0, 2.5, 11)
    ev[:, 2] = rng.uniform(0.25, 1.25, 11)
    ev[0, :3] = [5.0, 2.5, 1.25]; ev[1, :3] = [1.0, -2.0, 0.25]
    out = np.zeros((2, 11, 3))
    orc.orc_location_times(9, 7, 6, 1.0, -2.0, 0.5, 0.5, 0.75, 0.4, 2.0, 2, 11, 3, P(fields), P(ev), P(out))
    for p in range(2):
        for j in range(11):
            for k in range(3):
                assert out[p, j, k] == oloc.interpolate3d(fields[p, k], grid, ev[j, :3])
