"""GPU: the generalized R/T fundamental-mode kernel (mct_grt_batch,
mctomo_gb300/csrc/grt.cu) against the oracle's restatement of the
reference's RayleighModes / LoveModes (surfmodes/surfmodes.f90:185-303) on
layered columns with low-velocity layers. Both evaluate the reference's
arithmetic in FP64 without fused multiply-add and differ only in the last
bits of exp, sin and cos: every column gets the same ierr, and the phase
and group velocities agree within 1e-9 km/s except at the rare frequencies
where the scan for the first sign change sees a near-touching crossing on
one side only; there the GPU's velocity must still be a root of the
oracle's secular function. Also the routing of mct_surfmodes: a column with
a low-velocity layer slower than the top layer goes to the generalized R/T
search, one without to surfdisp96."""
import ctypes

import numpy as np
import pytest

from mctomo_gb300 import forward, synthetic
from test_grt_oracle import grt

pytestmark = pytest.mark.gpu
P = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731


def lvl_columns(orc, seed, n):
    rng = np.random.default_rng(seed)
    nl, thk, vp, vs, rho = synthetic.layered_columns(rng, 8 * n, nl_range=(12, 40), lvl_prob=0.1)
    thk, vp, vs, rho = (x.astype(np.float64) for x in (thk, vp, vs, rho))
    keep = []
    for c in range(len(nl)):
        k = nl[c]
        if orc.orc_grt_nlvls1(int(k), P(np.ascontiguousarray(thk[c, :k])), P(np.ascontiguousarray(vp[c, :k])),
                              P(np.ascontiguousarray(vs[c, :k])), P(np.ascontiguousarray(rho[c, :k])), 1) > 0:
            keep.append(c)
        if len(keep) == n:
            break
    keep = np.array(keep)
    return nl[keep], thk[keep], vp[keep], vs[keep], rho[keep]


def is_root(orc, col, mt, f, c, tol, smin):
    """c is a zero of the oracle's secular function at frequency f: a sign
    change within 4 tol of c, or bisecim's acceptance test at c
    (|f|^2 + |imf|^2 < 2 smin^2, util.f90:90-167)."""
    P_ = [np.ascontiguousarray(x) for x in col]
    im = np.zeros(1)
    ev = lambda x: orc.orc_grt_secfun(len(P_[0]), P(P_[0]), P(P_[1]), P(P_[2]), P(P_[3]), mt, f, x, P(im))  # noqa: E731
    if ev(c - 4 * tol) * ev(c + 4 * tol) <= 0:
        return True
    v = ev(c)
    return v * v + im[0] * im[0] < 2 * smin * smin


@pytest.mark.parametrize("mt", [1, 0])
@pytest.mark.parametrize("order", ["ascending", "descending"])
def test_grt_batch_matches_the_oracle(orc, gpulib, mt, order):
    # The search is a scan for the first sign change of the secular function
    # followed by bisection; where the function nearly touches zero between
    # two trial velocities, the last bits of exp / sin / cos (CUDA's against
    # the host's) can decide whether a crossing is seen, and both searches
    # then return roots of different branches. Those entries must be roots
    # of the oracle's own secular function and stay rare; all others agree
    # within 1e-9 km/s.
    nl, thk, vp, vs, rho = lvl_columns(orc, 11 + mt, 24)
    freqs = 1.0 / np.geomspace(0.2, 20.0, 20)
    if order == "ascending":
        freqs = freqs[::-1].copy()
    paras = forward.modes_para(mt, 1, tol=1e-6, dc=1e-3)
    ph, gr, ierr, nev = forward.grt_batch(nl, thk, vp, vs, rho, freqs, paras)
    assert nev > 0
    entries = flips = 0
    for c in range(len(nl)):
        k = nl[c]
        col = (thk[c, :k], vp[c, :k], vs[c, :k], rho[c, :k])
        e, eph, egr, ne = grt(orc, *col, freqs, mt)
        assert ierr[c] == e, (c, ierr[c], e)
        for i in range(len(freqs)):
            entries += 1
            if abs(ph[c, i] - eph[i]) <= 1e-9 and abs(gr[c, i] - egr[i]) <= 1e-9:
                continue
            flips += 1
            if abs(ph[c, i] - eph[i]) > 1e-9:
                n = len(freqs)
                tol = 1e-6 + (n - i) * 9e-6 / n
                smin = float(np.float32(1e-3)) + i * (float(np.float32(5e-3)) - float(np.float32(1e-3))) / n
                assert is_root(orc, col, mt, freqs[i], ph[c, i], tol, smin), (c, i, ph[c, i], eph[i])
    assert flips <= 0.02 * entries, (flips, entries)
    assert np.sum(ierr == 0) >= len(nl) // 2


def test_surfmodes_routes_low_velocity_layers(orc, gpulib):
    d = np.array([1.0, 1.0, 2.0, 0.0])
    vs = np.array([1.5, 1.0, 2.0, 3.0])            # layer 2 slower than the top: generalized R/T
    vp, rho = vs * 1.73, np.full(4, 2.5)
    freqs = np.array([2.0, 1.0, 0.5, 0.25])
    ph, gr, ierr = forward.surfmodes(d, vp, vs, rho, freqs, 1, 1, 1e-3)
    e, eph, egr, _ = grt(orc, d, vp, vs, rho, freqs, 1, tol=1e-6, dc=1e-3)
    assert ierr == e
    np.testing.assert_allclose(ph, eph, rtol=0, atol=1e-9)
    np.testing.assert_allclose(gr, egr, rtol=0, atol=1e-9)
    # no low-velocity layer: surfdisp96 on the REAL*4 model, as before
    vs2 = np.array([1.0, 1.5, 2.0, 3.0])
    ph2, _, ierr2 = forward.surfmodes(d, vs2 * 1.73, vs2, rho, freqs, 1, 0, 1e-3)
    cp, cg = np.zeros(4), np.zeros(4)
    f32 = lambda a: np.ascontiguousarray(a, np.float32)  # noqa: E731
    orc.orc_surfdisp96(P(f32(d)), P(f32(vs2 * 1.73)), P(f32(vs2)), P(f32(rho)), 4, 2, 1, 0, 4,
                       P(np.ascontiguousarray(1.0 / freqs)), 1e-3, P(cp), P(cg), None)
    assert ierr2 == 0
    np.testing.assert_allclose(ph2, cp, rtol=0, atol=1e-5)


def test_fluid_and_bad_columns_are_flagged(gpulib):
    nl = np.array([4, 1, 4], np.int32)
    thk = np.tile([1.0, 1.0, 1.0, 0.0], (3, 1))
    vs = np.tile([1.5, 1.0, 2.0, 3.0], (3, 1))
    vs[2, 0] = 0.0                                  # a fluid layer
    vp, rho = vs * 1.73 + 1.5 * (vs == 0), np.full((3, 4), 2.5)
    ph, gr, ierr, _ = forward.grt_batch(np.array([4, 4, 4], np.int32), thk, vp, vs, rho, np.array([1.0]),
                                        forward.modes_para(1, 1))
    assert ierr[2] == -2
    from mctomo_gb300 import MctError
    with pytest.raises(MctError):
        forward.grt_batch(nl, thk, vp, vs, rho, np.array([1.0]), forward.modes_para(1, 1))
