"""CPU: the oracle's 2D travel-time reductions (mcmc2d/likelihood_dd.F90
body_likelihood after modrays and body_noise_likelihood) against a direct
transcription of the same sums on a small case, including the reference's
quirks: the swapped-index differential-time test, the REAL*4 eps, PI2 and
nrays/2.0, and the INTEGER differential sigma log-sum of the noise step."""
import ctypes
import math

import numpy as np

P = lambda a: None if a is None else a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
PI2 = float(np.float32(6.283185))
EPS = float(np.float32(0.000000001))


def case(rng, nsrc=4, nrev=5):
    pt = rng.uniform(1.0, 4.0, (nsrc, nrev))
    obs = pt.reshape(-1) + 0.05 * rng.standard_normal(nsrc * nrev)
    rays = (rng.random(nsrc * nrev) < 0.8).astype(np.int32)
    sig = rng.uniform(0.02, 0.08, nsrc * nrev)
    ndd = nsrc * (nsrc - 1) // 2
    dtime = rng.normal(0, 0.3, (ndd, nrev))     # [dd][k] = column-major (nrev, ndd)
    dtime[rng.random(dtime.shape) < 0.3] = 0.0
    dcc = rng.uniform(0.2, 0.9, (ndd, nrev))
    return pt, obs, rays, sig, dtime, dcc


def expected(pt, obs, rays, sig, sigdep, datatype, dtime, dcc, ndtime, n0, n1, nrays, noise=False, srdist=None,
             int_sum=None):
    int_sum = noise if int_sum is None else int_sum
    nsrc, nrev = pt.shape
    flat_dt = dtime.reshape(-1)                  # column-major (nrev, ndd) storage
    if noise:
        sigma = n0[0] * srdist + n1[0]
    else:
        sigma = n0[0] * pt.reshape(-1) + n1[0] if sigdep else sig.copy()
    like = mis = umis = 0.0
    for n in range(nsrc * nrev):
        j, k = divmod(n, nrev)
        if rays[n] == 1:
            r = pt[j, k] - obs[n]
            like += r * r / (2 * sigma[n] ** 2); mis += r * r / sigma[n] ** 2; umis += r * r
        else:
            sigma[n] = 1.0
    like = like + sum(math.log(s) for s in sigma) + float(np.float32(nrays) / np.float32(2.0)) * math.log(PI2)
    if datatype == 1:
        sd = 0 if int_sum else 0.0
        dd = 0
        for i in range(nsrc):
            for j in range(i + 1, nsrc):
                for k in range(nrev):
                    if abs(flat_dt[dd + k * nrev]) > EPS:           # dat%dtime(ddindex,k,1)
                        r = (pt[j, k] - pt[i, k]) - dtime[dd, k]
                        s2 = n0[1] * (1 - dcc[dd, k]) + n1[1]
                        like += r * r / (2 * s2 * s2); mis += r * r / (s2 * s2); umis += r * r
                        sd = int(sd + math.log(s2)) if int_sum else sd + math.log(s2)
                dd += 1
        like = like + sd + float(np.float32(ndtime) / np.float32(2.0)) * math.log(PI2)
    return like, mis, umis


def test_tt2d_misfit_matches_transcription(orc):
    rng = np.random.default_rng(5)
    pt, obs, rays, sig, dtime, dcc = case(rng)
    nsrc, nrev = pt.shape
    for sigdep in (0, 1):
        for datatype in (0, 1):
            n0 = np.array([0.01, 0.02]); n1 = np.array([0.03, 0.01])
            out = np.zeros(3)
            st = orc.orc_tt2d_misfit(nsrc, nrev, P(np.ascontiguousarray(pt)), P(obs), P(sig), P(rays), sigdep,
                                     datatype, P(dtime), P(dcc), 17, P(n0), P(n1), int(rays.sum()), P(out))
            exp = expected(pt, obs, rays, sig, sigdep, datatype, dtime, dcc, 17, n0, n1, int(rays.sum()))
            assert st == 0
            np.testing.assert_allclose(out, exp, rtol=1e-12)


def test_tt2d_noise_integer_logsum(orc):
    rng = np.random.default_rng(6)
    pt, obs, rays, sig, dtime, dcc = case(rng)
    nsrc, nrev = pt.shape
    srd = rng.uniform(1.0, 10.0, nsrc * nrev)
    n0 = np.array([0.005, 0.02]); n1 = np.array([0.02, 0.03])
    out = np.zeros(2)
    st = orc.orc_tt2d_noise(nsrc, nrev, P(np.ascontiguousarray(pt)), P(obs), P(rays), P(srd), 1, P(dtime),
                            P(dcc), 17, P(n0), P(n1), int(rays.sum()), P(out))
    exp = expected(pt, obs, rays, sig, 0, 1, dtime, dcc, 17, n0, n1, int(rays.sum()), noise=True, srdist=srd)
    assert st == 0
    np.testing.assert_allclose(out, exp[:2], rtol=1e-12)
    # the integer sum differs from the real one: the quirk is exercised
    real = expected(pt, obs, rays, sig, 0, 1, dtime, dcc, 17, n0, n1, int(rays.sum()), noise=True, srdist=srd,
                    int_sum=False)
    assert abs(real[0] - exp[0]) > 0.5
    # zero sigma anywhere (even on a pair without data) is the fatal error
    n1z = np.array([0.0, 0.03])
    assert orc.orc_tt2d_noise(nsrc, nrev, P(np.ascontiguousarray(pt)), P(obs), P(rays), P(np.zeros_like(srd)), 1,
                              P(dtime), P(dcc), 17, P(np.array([0.0, 0.02])), P(n1z), 5, P(out)) == 8
