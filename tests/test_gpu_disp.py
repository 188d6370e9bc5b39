"""GPU parity: surfdisp96 dispersion kernel vs the CPU restatement.

Tolerance: phase velocity within 1e-5 km/s (the stated accuracy bound); the
outputs are REAL*4-rounded roots, so in practice they agree to the last
REAL*4 bit except where CUDA's and the host's sin/cos/exp differ by an ulp
right at a sign decision. Group velocity (REAL*4 finite difference in the
reference) within 1e-4 km/s.
"""
import ctypes

import numpy as np
import pytest

from mctomo_gb300 import surfdisp96, surfdisp_batch, surfdisp_mmodes, surfmodes, MctError, synthetic

pytestmark = pytest.mark.gpu
P = lambda a: None if a is None else a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
PHASE_TOL = 1e-5
GROUP_TOL = 1e-4


def monotone_columns(rng, ncol, nl_max=31):
    nl = rng.integers(3, nl_max + 1, ncol).astype(np.int32)
    thk = np.zeros((ncol, nl_max), np.float32)
    vs = np.zeros((ncol, nl_max), np.float32)
    for c in range(ncol):
        n = nl[c]
        v = np.sort(rng.uniform(0.3, 2.5, n))
        vs[c, :n] = v; vs[c, n:] = v[-1]
        thk[c, :n - 1] = rng.uniform(0.05, 0.8, n - 1)
    vp = (vs * np.float32(1.73)).astype(np.float32)
    rho = np.full_like(vs, 2.0)
    return nl, thk, vp, vs, rho


def oracle_cols(orc, nl, thk, vp, vs, rho, per, iwave, igr, mode=1, multi=False):
    ncol = len(nl)
    cp = np.zeros((ncol, mode, per.size)); cg = np.zeros((ncol, mode, per.size))
    ierr = np.zeros(ncol, np.int32)
    fn = orc.orc_surfdisp_mmodes if multi else orc.orc_surfdisp96
    for c in range(ncol):
        a = [np.ascontiguousarray(x[c, :nl[c]]) for x in (thk, vp, vs, rho)]
        o1 = np.zeros(mode * per.size); o2 = np.zeros(mode * per.size)
        ierr[c] = fn(*[P(x) for x in a], int(nl[c]), iwave, mode, igr, per.size, P(per), 0.001, P(o1), P(o2), None)
        cp[c] = o1.reshape(mode, per.size); cg[c] = o2.reshape(mode, per.size)
    return cp, cg, ierr


@pytest.mark.parametrize("iwave,igr", [(2, 0), (1, 0), (2, 1), (1, 1)])
def test_surfdisp_batch_matches_oracle(orc, gpulib, iwave, igr):
    rng = np.random.default_rng(100 + iwave * 10 + igr)
    nl, thk, vp, vs, rho = monotone_columns(rng, 96)
    per = np.geomspace(0.5, 5.0, 20)
    cp, cg, ierr, cnt = surfdisp_batch(nl, thk, vp, vs, rho, per, iwave, igr, 0.001)
    ecp, ecg, eierr = oracle_cols(orc, nl, thk, vp, vs, rho, per, iwave, igr)
    np.testing.assert_array_equal(ierr, eierr)
    ok = eierr == 0
    assert ok.sum() > 48
    assert np.max(np.abs(cp[ok] - ecp[ok])) <= PHASE_TOL
    if igr:
        assert np.max(np.abs(cg[ok] - ecg[ok])) <= GROUP_TOL
    assert cnt[0] > 0


def test_fp32_bracketing_gives_the_fp64_roots(gpulib):
    rng = np.random.default_rng(7)
    nl, thk, vp, vs, rho = monotone_columns(rng, 128)
    per = np.geomspace(0.5, 5.0, 20)
    a = surfdisp_batch(nl, thk, vp, vs, rho, per, 2, 0, 0.001, precision=0)
    b = surfdisp_batch(nl, thk, vp, vs, rho, per, 2, 0, 0.001, precision=1)
    np.testing.assert_array_equal(a[2], b[2])
    np.testing.assert_array_equal(a[0], b[0])
    assert b[3][0] < a[3][0] * 0.7   # the bracketing scans moved to FP32


def test_mmodes_and_single_column_entry_points(orc, gpulib):
    rng = np.random.default_rng(21)
    nl, thk, vp, vs, rho = monotone_columns(rng, 12, nl_max=15)
    per = np.geomspace(0.3, 8.0, 12)
    for c in range(12):
        n = nl[c]
        args = [x[c, :n] for x in (thk, vp, vs, rho)]
        cp, cg, ierr = surfdisp96(*args, iwave=2, igr=0, t=per, dphase=0.001)
        e = oracle_cols(orc, nl[c:c + 1], thk[c:c + 1], vp[c:c + 1], vs[c:c + 1], rho[c:c + 1], per, 2, 0)
        assert ierr == e[2][0]
        if ierr == 0:
            assert np.max(np.abs(cp - e[0][0, 0])) <= PHASE_TOL
        mcp, mcg, mierr = surfdisp_mmodes(*args, iwave=1, mode=2, igr=1, t=per, dphase=0.001)
        e2 = oracle_cols(orc, nl[c:c + 1], thk[c:c + 1], vp[c:c + 1], vs[c:c + 1], rho[c:c + 1], per, 1, 1, mode=2, multi=True)
        assert mierr == e2[2][0]
        good = e2[0][0] > 0
        assert np.max(np.abs(mcp[good] - e2[0][0][good]), initial=0) <= PHASE_TOL


def test_surfmodes_routes_lvl_columns_to_grt(orc, gpulib):
    # a layer slower than the top layer: the generalized R/T search, as the
    # reference's surfmodes routes it (surfmodes.f90:39-108); under a fluid
    # layer that path (the Stoneley mode) is not built and is refused
    from test_grt_oracle import grt
    thick = np.array([1.0, 1.0, 1.0, 0.0])
    vs = np.array([1.0, 0.6, 1.5, 2.0])
    vp = vs * 1.73
    rho = np.full(4, 2.0)
    freqs = 1.0 / np.geomspace(0.5, 5, 5)
    ph, gr, ierr = surfmodes(thick, vp, vs, rho, freqs, 1, 0, 0.001)
    e, eph, _, _ = grt(orc, thick, vp, vs, rho, freqs, 1, pg=0)
    assert ierr == e
    np.testing.assert_allclose(ph, eph, rtol=0, atol=1e-9)
    # water over a solid whose second layer is slower than the first
    with pytest.raises(MctError) as ei:
        surfmodes(thick, np.array([1.5, 1.73, 1.04, 3.46]), np.array([0.0, 1.0, 0.6, 2.0]), rho, freqs, 1, 0, 0.001)
    assert ei.value.code == -5
    ph, gr, ierr = surfmodes(thick, vp, np.array([1.0, 1.2, 1.5, 2.0]), rho, freqs, 1, 0, 0.001)
    assert ierr == 0 and np.all(ph > 0.8) and np.all(ph < 2.0)


def test_lvl_columns_of_the_precision_study_run_on_surfdisp96(orc, gpulib):
    # columns with low-velocity layers (config 4): reported separately, still
    # compared with the surfdisp96 restatement
    rng = np.random.default_rng(33)
    nl, thk, vp, vs, rho = synthetic.layered_columns(rng, 64, nl_range=(12, 40))
    per = np.geomspace(0.2, 20.0, 30)
    cp, cg, ierr, _ = surfdisp_batch(nl, thk, vp, vs, rho, per, 2, 1, 0.001, precision=1)
    ecp, ecg, eierr = oracle_cols(orc, nl, thk, vp, vs, rho, per, 2, 1)
    same = ierr == eierr
    assert same.mean() > 0.95
    ok = (ierr == 0) & (eierr == 0)
    assert np.max(np.abs(cp[ok] - ecp[ok])) <= PHASE_TOL


@pytest.mark.parametrize("iwave,precision", [(2, 1), (1, 1), (2, 0)])
def test_lanes_evaluating_ahead_give_the_same_roots(gpulib, iwave, precision):
    # idle lanes evaluate the next trial velocities of long bracketing scans,
    # and the columns run in order of layer count; every root, group
    # velocity, error flag must be the same bits as with each column
    # scanning alone in batch order (multimode, group, columns of the
    # precision study with low-velocity layers, which give the long scans)
    rng = np.random.default_rng(44 + iwave + precision)
    nl, thk, vp, vs, rho = synthetic.layered_columns(rng, 256, nl_range=(12, 40), lvl_prob=0.1)
    per = np.geomspace(0.2, 20.0, 60)
    old = gpulib.mct_debug_disp_share(0)       # no lookahead, columns in batch order
    try:
        a = surfdisp_batch(nl, thk, vp, vs, rho, per, iwave, 1, 0.001, mode=2, multimode=True, precision=precision)
        gpulib.mct_debug_disp_share(3)           # lookahead, columns by layer count
        b = surfdisp_batch(nl, thk, vp, vs, rho, per, iwave, 1, 0.001, mode=2, multimode=True, precision=precision)
    finally:
        gpulib.mct_debug_disp_share(old)
    np.testing.assert_array_equal(a[2], b[2])
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])
    assert b[3] == a[3]      # the searches used the same evaluations (values ahead not reached are not counted)


@pytest.mark.parametrize("iwave", [2, 1])
def test_fp64_search_makes_the_reference_evaluations(orc, gpulib, iwave):
    # precision 0 runs the reference's own search: the number of period-
    # equation evaluations it used equals the oracle's count for the same
    # columns (multimode, group, columns with low-velocity layers), up to
    # the odd Neville step: CUDA's sin / cos / exp and the host's can differ
    # in the last bit, which can move a convergence test by one step (seen:
    # 1 evaluation in 447,853 for Love, none for Rayleigh)
    rng = np.random.default_rng(55 + iwave)
    nl, thk, vp, vs, rho = synthetic.layered_columns(rng, 48, nl_range=(12, 40), lvl_prob=0.1)
    per = np.geomspace(0.2, 20.0, 60)
    cp, cg, ierr, cnt = surfdisp_batch(nl, thk, vp, vs, rho, per, iwave, 1, 0.001, mode=2, multimode=True,
                                       precision=0)
    total = 0
    for c in range(len(nl)):
        a = [np.ascontiguousarray(x[c, :nl[c]]) for x in (thk, vp, vs, rho)]
        o1 = np.zeros(120); o2 = np.zeros(120); n = np.zeros(1, np.int64)
        orc.orc_surfdisp_mmodes(*[P(x) for x in a], int(nl[c]), iwave, 2, 1, 60, P(per), 0.001, P(o1), P(o2), P(n))
        total += int(n[0])
    assert cnt[1] == 0
    assert abs(int(cnt[0]) - total) <= max(2, total // 100000)
    _, _, _, cnt1 = surfdisp_batch(nl, thk, vp, vs, rho, per, iwave, 1, 0.001, mode=2, multimode=True, precision=1)
    assert cnt1[0] < total // 2 and cnt1[1] > 0
