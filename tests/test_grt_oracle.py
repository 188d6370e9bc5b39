"""CPU: the oracle's generalized R/T fundamental-mode search (oracle/grt.cpp,
the reference's RayleighModes / LoveModes, surfmodes/surfmodes.f90:185-303)
against known answers:

* Love waves in a layer over a half-space: the closed-form period equation
  tan(w H q1) = mu2 q2' / (mu1 q1);
* Love waves in multilayer columns: an independent Thomson-Haskell
  propagator (numpy, complex arithmetic) solved with brentq;
* Rayleigh waves in a homogeneous medium: the Rayleigh function's root, the
  same at every frequency (phase = group);
* Rayleigh and Love waves in layered columns without a low-velocity layer,
  at frequencies whose root lies below the top layer's shear velocity: the
  surfdisp96 oracle (phase only, igr = 0).

Each root is within the tolerance the search runs at (tolmax = 1e-5 km/s).
Also the routing count nlvls1 (setup_grt, surfmodes.f90:320-450)."""
import ctypes

import numpy as np
import pytest
from scipy.optimize import brentq

P = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
TOL = 1e-6


def grt(orc, thk, vp, vs, rho, freqs, mt, pg=1, tol=TOL, dc=1e-3):
    a = [np.ascontiguousarray(x, dtype=np.float64) for x in (thk, vp, vs, rho, freqs)]
    n, m = len(a[0]), len(a[4])
    ph, gr, ne = np.zeros(m), np.zeros(m), np.zeros(1, np.int64)
    e = orc.orc_grt_modes(n, P(a[0]), P(a[1]), P(a[2]), P(a[3]), m, P(a[4]), mt, pg, tol, 10 * tol,
                          float(np.float32(1e-3)), float(np.float32(5e-3)), dc, dc, dc, P(ph), P(gr), P(ne))
    return e, ph, gr, int(ne[0])


def love_haskell(c, f, h, b, r):
    """Love-wave period equation by the propagator matrix of (v, tau) from
    the free surface to the half-space: tau + mu_n nu_n v = 0."""
    k = 2 * np.pi * f / c
    y = np.array([1.0 + 0j, 0j])
    for j in range(len(h) - 1):
        mu = r[j] * b[j] ** 2
        nu = k * np.sqrt(complex(1 - c * c / b[j] ** 2))
        ch, sh = np.cosh(nu * h[j]), np.sinh(nu * h[j])
        y = np.array([[ch, sh / (mu * nu)], [mu * nu * sh, ch]]) @ y
    mu = r[-1] * b[-1] ** 2
    return (y[1] + mu * k * np.sqrt(1 - c * c / b[-1] ** 2) * y[0]).real


def lowest_root(fn, lo, hi, n=20001):
    cs = np.linspace(lo, hi, n)
    v = np.array([fn(x) for x in cs])
    i = np.where(v[:-1] * v[1:] < 0)[0]
    return brentq(fn, cs[i[0]], cs[i[0] + 1], xtol=1e-14)


def test_love_layer_over_halfspace(orc):
    H, b1, b2, r1, r2 = 2.0, 2.0, 3.5, 2.2, 2.6
    m1, m2 = r1 * b1 ** 2, r2 * b2 ** 2
    freqs = np.array([0.1, 0.2, 0.5, 1.0, 2.0])

    def period_eq(c, f):
        q = np.sqrt(1 / b1 ** 2 - 1 / c ** 2)
        return np.sin(2 * np.pi * f * H * q) * m1 * q - np.cos(2 * np.pi * f * H * q) * m2 * np.sqrt(
            1 / c ** 2 - 1 / b2 ** 2)
    e, ph, gr, ne = grt(orc, [H, 0.0], [b1 * 1.8, b2 * 1.8], [b1, b2], [r1, r2], freqs, 0)
    assert e == 0 and ne > 0
    for f, c in zip(freqs, ph):
        exact = lowest_root(lambda x: period_eq(x, f), b1 * (1 + 1e-9), b2 * (1 - 1e-9), 200001)
        assert abs(c - exact) < 1e-5, (f, c, exact)


@pytest.mark.parametrize("h,b", [([1.0, 2.0, 0.0], [1.0, 2.0, 3.0]), ([0.5, 0.5, 0.0], [1.0, 1.5, 2.0]),
                                 ([0.4, 0.8, 1.2, 0.0], [1.2, 1.6, 2.2, 3.0])])
def test_love_multilayer_against_haskell(orc, h, b):
    h, b = np.array(h), np.array(b)
    r = np.full(len(h), 2.5)
    freqs = np.array([0.1, 0.2, 0.5, 1.0, 2.0])
    e, ph, gr, _ = grt(orc, h, b * 1.75, b, r, freqs, 0)
    assert e == 0
    for f, c in zip(freqs, ph):
        exact = lowest_root(lambda x: love_haskell(x, f, h, b, r), b.min() * (1 + 1e-9), b[-1] * (1 - 1e-9))
        assert abs(c - exact) < 1e-5, (f, c, exact)


def test_rayleigh_homogeneous(orc):
    a, b = 3.0 * 1.732, 3.0
    cr = brentq(lambda c: (2 - c * c / b ** 2) ** 2 - 4 * np.sqrt(1 - c * c / a ** 2) * np.sqrt(1 - c * c / b ** 2),
                0.5 * b, 0.999 * b, xtol=1e-14)
    e, ph, gr, _ = grt(orc, [1.0, 0.0], [a, a], [b, b], [2.5, 2.5], np.array([0.1, 0.2, 0.5, 1.0, 2.0]), 1)
    assert e == 0
    assert np.max(np.abs(ph - cr)) < 1e-5
    assert np.max(np.abs(gr - cr)) < 1e-4      # finite difference over 0.005 Hz


@pytest.mark.parametrize("mt,iwave", [(1, 2), (0, 1)])
def test_layered_against_surfdisp96(orc, mt, iwave):
    # float-representable models, so surfdisp96's REAL*4 model is the same
    t4 = np.array([0.5, 1.0, 1.5, 0.0], np.float32)
    b4 = np.array([1.0, 1.5, 2.0, 2.75], np.float32)
    a4 = (b4 * 1.75).astype(np.float32)
    r4 = np.array([2.0, 2.25, 2.5, 2.75], np.float32)
    periods = np.array([0.25, 0.4, 0.6, 1.0])
    cp, cg = np.zeros(4), np.zeros(4)
    rc = orc.orc_surfdisp96(P(t4), P(a4), P(b4), P(r4), 4, iwave, 1, 0, 4, P(periods), 0.001, P(cp), P(cg), None)
    assert rc == 0
    e, ph, _, _ = grt(orc, t4.astype(float), a4.astype(float), b4.astype(float), r4.astype(float),
                      1.0 / periods, mt, pg=0)
    assert e == 0
    # surfdisp96 returns REAL*4 velocities
    np.testing.assert_allclose(ph, cp, atol=2e-5)


def test_routing_count(orc):
    d = np.array([1.0, 1.0, 1.0, 0.0])
    vs = np.array([1.5, 1.0, 2.0, 3.0])      # layer 2 is a low-velocity layer below a faster top
    vp = vs * 1.73
    rho = np.full(4, 2.5)
    assert orc.orc_grt_nlvls1(4, P(d), P(vp), P(vs), P(rho), 1) == 1
    vs2 = np.array([1.0, 1.5, 2.0, 3.0])
    assert orc.orc_grt_nlvls1(4, P(d), P(vs2 * 1.73), P(vs2), P(rho), 1) == 0
    vs3 = np.array([0.0, 1.5, 2.0, 3.0])     # fluid top: the Stoneley path is not restated
    assert orc.orc_grt_nlvls1(4, P(d), P(np.array([1.5, 2.6, 3.4, 5.2])), P(vs3), P(rho), 1) == -2


def test_route_matches_setup_grt(orc, gpulib):
    # mct_surfmodes_route (host code of the library) against the oracle's
    # setup_grt count, on synthetic study columns
    from mctomo_gb300 import forward, synthetic
    rng = np.random.default_rng(5)
    nl, thk, vp, vs, rho = synthetic.layered_columns(rng, 400, nl_range=(12, 40), lvl_prob=0.1)
    thk, vp, vs, rho = (np.ascontiguousarray(x, np.float64) for x in (thk, vp, vs, rho))
    for mt in (1, 0):
        route = forward.surfmodes_route(nl, vp, vs, mt)
        for c in range(len(nl)):
            k = int(nl[c])
            n = orc.orc_grt_nlvls1(k, P(np.ascontiguousarray(thk[c, :k])), P(np.ascontiguousarray(vp[c, :k])),
                                   P(np.ascontiguousarray(vs[c, :k])), P(np.ascontiguousarray(rho[c, :k])), mt)
            assert route[c] == (1 if n > 0 else 0), (c, route[c], n)
        assert 0 < np.sum(route == 1) < len(nl)


def test_roots_are_roots_of_the_surfdisp96_period_equations(orc):
    # On study columns with a low-velocity layer, the generalized R/T roots are
    # zeros of the Haskell-Thomson / Dunkin period equations that the
    # surfdisp96 oracle evaluates (dltar1 for Love, dltar4 for Rayleigh; an
    # independent formulation): a sign change within 4 tol. For Rayleigh this
    # holds below the top layer's shear velocity; above it the reference
    # brackets sign changes of the real part of its determinant and also
    # accepts points where that part is merely small, which are often not
    # roots (kept as the reference does; counted, not asserted).
    from mctomo_gb300 import synthetic
    rng = np.random.default_rng(21)
    nl, thk, vp, vs, rho = synthetic.layered_columns(rng, 300, nl_range=(12, 40), lvl_prob=0.1)
    freqs = 1.0 / np.geomspace(0.2, 20.0, 20)
    for mt, kk in ((0, 1), (1, 2)):
        hit = miss = cols = 0
        for c in range(len(nl)):
            n = int(nl[c])
            m4 = [np.ascontiguousarray(x[c, :n], np.float32) for x in (thk, vp, vs, rho)]
            m8 = [x.astype(np.float64) for x in m4]
            if orc.orc_grt_nlvls1(n, *[P(x) for x in m8], mt) <= 0:
                continue
            cols += 1
            if cols > 12:
                break
            _, ph, _, _ = grt(orc, *m8, freqs, mt)
            for i, (f, cv) in enumerate(zip(freqs, ph)):
                if cv <= 0 or (mt == 1 and cv >= m8[2][0]):
                    continue
                tol = 1e-6 + (len(freqs) - i) * 9e-6 / len(freqs)
                om = 2 * np.pi * f
                d = [orc.orc_dltar(om / x, om, kk, *[P(a) for a in m4], n) for x in (cv - 4 * tol, cv + 4 * tol)]
                if d[0] * d[1] <= 0:
                    hit += 1
                else:
                    miss += 1
        assert hit > 50 and miss <= 0.01 * (hit + miss), (mt, hit, miss)


def test_trial_list_beyond_the_reference_arrays(orc):
    # Two 200 km layers at 0.1 Hz: C_Interval_L would place (NN + 1) * 512
    # trial velocities, more than the reference's 20,000-entry arrays hold
    # (surfmodes/C_interval_L.f90:24-30); the column gets ierr 2 at once and
    # no secular evaluation. The Rayleigh search finds its root in the window
    # below vs1 and never builds the list.
    thk, vs = np.array([200.0, 200.0, 0.0]), np.array([1.5, 1.0, 3.0])
    vp, rho = vs * 1.73, np.full(3, 2.5)
    e, ph, gr, ne = grt(orc, thk, vp, vs, rho, np.array([0.1]), 0)
    assert e == 2 and ph[0] == 0 and ne == 0
    e, ph, gr, ne = grt(orc, thk, vp, vs, rho, np.array([0.1]), 1)
    assert e == 0 and ph[0] > 0
