"""GPU parity: fm2d travel times (modrays) vs the CPU restatement.

The GPU runs the reference's own marching order and heap, and the same
FP64 operations without FMA, so the travel times are expected to agree to
the last bit; the stated tolerance is 1e-9 s (far inside the 1e-4 s bound).
"""
import ctypes

import numpy as np
import pytest

from mctomo_gb300 import modrays, modrays_batch

pytestmark = pytest.mark.gpu
P = lambda a: None if a is None else a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
TOL = 1e-9
TT_MIXED_TOL = 1e-4


def voronoi_velv(rng, nvx, nvz, dx, dz, ncell, vrange):
    pts = rng.uniform(0, 1, (ncell, 2)) * [(nvx - 1) * dx, (nvz - 1) * dz]
    vals = rng.uniform(*vrange, ncell)
    X, Z = np.meshgrid(np.arange(nvx) * dx, np.arange(nvz) * dz, indexing="ij")
    d = (X[..., None] - pts[:, 0]) ** 2 + (Z[..., None] - pts[:, 1]) ** 2
    vel = vals[np.argmin(d, -1)]           # (nvx, nvz)
    ext = np.zeros((nvx + 2, nvz + 2))
    ext[1:-1, 1:-1] = vel
    ext[0] = ext[1]; ext[-1] = ext[-2]; ext[:, 0] = ext[:, 1]; ext[:, -1] = ext[:, -2]
    return ext


def oracle_modrays(orc, src, rev, srs, nvx, nvz, gox, goz, dx, dz, velv, gdx, gdz, asgr, sgdl, sgs, fom):
    nsrc, nrc = len(src), len(rev)
    tt = np.zeros((nsrc, nrc))
    sx, sz = np.ascontiguousarray(src[:, 0]), np.ascontiguousarray(src[:, 1])
    rx, rz = np.ascontiguousarray(rev[:, 0]), np.ascontiguousarray(rev[:, 1])
    rc = orc.orc_modrays(nsrc, P(sx), P(sz), nrc, P(rx), P(rz), P(np.ascontiguousarray(srs, np.int32)),
                         nvx, nvz, gox, goz, dx, dz, P(np.ascontiguousarray(velv)), gdx, gdz, asgr, sgdl,
                         sgs, fom, 0.5, P(tt), None)
    assert rc == 0
    return tt


def stations_perimeter(n, L, inset=0.5):
    """n stations equally spaced on a square inset from the domain edges.
    A source within one refined cell of a maximum edge makes the reference's
    refined pass stop before any refined node maps back onto the coarse grid,
    and the reference then reports stale memory as travel times; stations are
    kept away from the edges so the comparison is meaningful."""
    a, b = inset, L - inset
    side = b - a
    s = np.linspace(0, 4 * side, n, endpoint=False) + 0.37
    pts = []
    for v in s:
        if v < side: pts.append((a + v, a))
        elif v < 2 * side: pts.append((b, a + v - side))
        elif v < 3 * side: pts.append((b - (v - 2 * side), b))
        else: pts.append((a, b - (v - 3 * side)))
    return np.array(pts)


@pytest.mark.parametrize("asgr,fom,sgdl,sgs", [(1, 1, 5, 10), (1, 0, 4, 8), (0, 1, 4, 8), (0, 0, 4, 8)])
def test_modrays_2d_config_shape_matches_oracle(orc, gpulib, asgr, fom, sgdl, sgs):
    # 10 x 10 km, 51 x 51 grid, 16 stations on the perimeter, all pairs
    rng = np.random.default_rng(asgr * 10 + fom)
    nvx = nvz = 51
    dx = dz = 0.2
    velv = voronoi_velv(rng, nvx, nvz, dx, dz, 20, (2.0, 4.0))
    st = stations_perimeter(16, 10.0)
    srs = 1 - np.eye(16, dtype=np.int32)
    got = modrays(st, st, srs, nvx, nvz, 0.0, 0.0, dx, dz, velv, asgr=asgr, sgdl=sgdl, sgs=sgs, fom=fom)
    exp = oracle_modrays(orc, st, st, srs, nvx, nvz, 0.0, 0.0, dx, dz, velv, 1, 1, asgr, sgdl, sgs, fom)
    m = srs == 1
    assert np.max(np.abs(got[m] - exp[m])) <= TOL


def test_modrays_batch_surface_shape_matches_oracle(orc, gpulib):
    # 41 x 41 phase-velocity maps, 12 stations, upper-triangle paths
    rng = np.random.default_rng(4)
    nvx = nvz = 41
    dx = dz = 1.0
    nmaps = 6
    velv = np.stack([voronoi_velv(rng, nvx, nvz, dx, dz, 30, (0.4, 2.2)) for _ in range(nmaps)])
    st = rng.uniform(2.0, 38.0, (12, 2))
    srs = np.triu(np.ones((12, 12), np.int32), 1)
    got = modrays_batch(st, st, srs, nvx, nvz, 0.0, 0.0, dx, dz, velv, sgdl=4, sgs=8)
    for mp in range(nmaps):
        exp = oracle_modrays(orc, st, st, srs, nvx, nvz, 0.0, 0.0, dx, dz, velv[mp], 1, 1, 1, 4, 8, 1)
        m = srs == 1
        assert np.max(np.abs(got[mp][m] - exp[m])) <= TOL


@pytest.mark.parametrize("cap", [16, 64])
def test_modrays_heap_overflow_pass_matches_oracle(orc, gpulib, cap):
    # a refined-stage heap far smaller than the narrow band: nearly every
    # solve overflows the first pass and is redone with a full heap
    rng = np.random.default_rng(5)
    nvx = nvz = 41
    nmaps = 3
    velv = np.stack([voronoi_velv(rng, nvx, nvz, 1.0, 1.0, 30, (0.4, 2.2)) for _ in range(nmaps)])
    st = rng.uniform(2.0, 38.0, (10, 2))
    srs = np.triu(np.ones((10, 10), np.int32), 1)
    base = modrays_batch(st, st, srs, nvx, nvz, 0.0, 0.0, 1.0, 1.0, velv, sgdl=4, sgs=8, precision=1)
    gpulib.mct_debug_fm2d_heap_cap(cap)
    try:
        got = modrays_batch(st, st, srs, nvx, nvz, 0.0, 0.0, 1.0, 1.0, velv, sgdl=4, sgs=8)
        got_df = modrays_batch(st, st, srs, nvx, nvz, 0.0, 0.0, 1.0, 1.0, velv, sgdl=4, sgs=8, precision=1)
    finally:
        gpulib.mct_debug_fm2d_heap_cap(0)
    m = srs == 1
    for mp in range(nmaps):
        exp = oracle_modrays(orc, st, st, srs, nvx, nvz, 0.0, 0.0, 1.0, 1.0, velv[mp], 1, 1, 1, 4, 8, 1)
        assert np.max(np.abs(got[mp][m] - exp[m])) <= TOL
    np.testing.assert_array_equal(got_df, base)


def test_modrays_homogeneous_close_to_straight_line(gpulib):
    nvx = nvz = 41
    velv = np.full((nvx + 2, nvz + 2), 3.0)
    src = np.array([[3.3, 4.1]])
    rev = np.array([[8.7, 1.2], [1.1, 9.3], [9.6, 9.6]])
    tt = modrays(src, rev, np.ones((1, 3), np.int32), nvx, nvz, 0.0, 0.0, 0.25, 0.25, velv)
    exact = np.hypot(rev[:, 0] - 3.3, rev[:, 1] - 4.1) / 3.0
    assert np.all(np.abs(tt[0] - exact) / exact < 0.01)


def test_modrays_source_outside_is_an_error(gpulib):
    from mctomo_gb300 import MctError
    velv = np.full((43, 43), 3.0)
    with pytest.raises(MctError) as ei:
        modrays(np.array([[50.0, 1.0]]), np.array([[1.0, 1.0]]), np.ones((1, 1), np.int32), 41, 41, 0., 0.,
                0.25, 0.25, velv)
    assert ei.value.code == -4


def test_modrays_double_float_within_tolerance(orc, gpulib):
    # double-float updates (~2^-48 relative): every path within 1e-4 s of the
    # FP64 path (in practice ~1e-12 s)
    rng = np.random.default_rng(8)
    nvx = nvz = 41
    velv = np.stack([voronoi_velv(rng, nvx, nvz, 1.0, 1.0, 40, (0.4, 2.2)) for _ in range(4)])
    st = rng.uniform(2.0, 38.0, (20, 2))
    srs = np.triu(np.ones((20, 20), np.int32), 1)
    exact = modrays_batch(st, st, srs, nvx, nvz, 0.0, 0.0, 1.0, 1.0, velv, sgdl=4, sgs=8, precision=0)
    dfl = modrays_batch(st, st, srs, nvx, nvz, 0.0, 0.0, 1.0, 1.0, velv, sgdl=4, sgs=8, precision=1)
    m = np.broadcast_to(srs == 1, exact.shape)
    assert np.max(np.abs(dfl[m] - exact[m])) <= TT_MIXED_TOL


@pytest.mark.parametrize("precision", [2])
def test_modrays_fixed_point_error_statistics(orc, gpulib, precision):
    # FP32 updates on fixed-point times perturb times by ~1e-7 s, which can
    # flip the acceptance order of near-tied nodes; fm2d's mixed-order
    # stencils then switch and single paths move by up to ~1e-2 s. This is
    # the approximate mode: 99% of paths within 1e-4 s, all within 5e-2 s.
    rng = np.random.default_rng(8)
    nvx = nvz = 41
    velv = np.stack([voronoi_velv(rng, nvx, nvz, 1.0, 1.0, 40, (0.4, 2.2)) for _ in range(4)])
    st = rng.uniform(2.0, 38.0, (20, 2))
    srs = np.triu(np.ones((20, 20), np.int32), 1)
    exact = modrays_batch(st, st, srs, nvx, nvz, 0.0, 0.0, 1.0, 1.0, velv, sgdl=4, sgs=8, precision=0)
    mixed = modrays_batch(st, st, srs, nvx, nvz, 0.0, 0.0, 1.0, 1.0, velv, sgdl=4, sgs=8, precision=precision)
    m = np.broadcast_to(srs == 1, exact.shape)
    err = np.abs(mixed[m] - exact[m])
    assert np.quantile(err, 0.99) <= TT_MIXED_TOL
    assert err.max() <= 5e-2


def test_exact_sqrt_matches_library_sqrt_bit_for_bit(gpulib):
    # the FP64 update's square root runs on the integer and FP32 pipes; it
    # must give the library sqrt's bits on every input: 2^26 inputs over the
    # whole exponent range, exact and near-exact squares, squares of
    # midpoints between doubles (the hardest rounding cases), and special
    # values (zero, subnormal, infinite, NaN, negative)
    out = (ctypes.c_ulonglong * 3)()
    for seed in (1, 2):
        assert gpulib.mct_debug_exact_sqrt_check(ctypes.c_ulonglong(1 << 26), ctypes.c_ulonglong(seed), out) == 0
        assert out[0] == 0, "first differing input bits: %#x" % out[2]
