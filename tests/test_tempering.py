"""CPU: parallel tempering (mct_pt_*, mct_mcmc_accept_tempered) against the
oracle's restatement of mcmc_pt's choose_t1 / choose_t2 / do_tempering
(src/mcmc_loc2.f90:2148-2280) with its own MT19937, step for step: the
chosen chains, the swap decisions, the chains' temperatures and ladder
positions, and the draws taken from the stream."""
import ctypes
import math

import numpy as np
import pytest

from mctomo_gb300 import lib, sampler
from oracle import tempering as otp

LADDER = [1.0, 1.0, 1.0, 1.6, 2.5, 4.0, 6.3, 10.0]


class _Rng:
    def __init__(self, seed):
        self.rng = ctypes.c_void_p()
        assert lib().mct_rng_create(seed, ctypes.byref(self.rng)) == 0

    def count(self):
        return lib().mct_rng_count(self.rng)

    def close(self):
        lib().mct_rng_destroy(self.rng)


def test_oracle_mt19937_known_answer():
    mt = otp.Mt(5489)
    assert mt.u32() == 3499211612
    for _ in range(9998):
        mt.u32()
    assert mt.u32() == 4123659995


@pytest.mark.parametrize("jump_type", [0, 1, 2])
def test_tempering_matches_oracle(jump_type):
    seed = 1234 + jump_type
    pt = sampler.Tempering(LADDER, number_of_1s=3, jump_type=jump_type)
    r = _Rng(seed)
    mt = otp.Mt(seed)
    draws = [0]
    unirand = mt.unirand

    def counted():
        draws[0] += 1
        return unirand()
    mt.unirand = counted
    values, indices = list(LADDER), list(range(1, len(LADDER) + 1))
    like = np.random.default_rng(seed).uniform(100.0, 140.0, (400, len(LADDER)))
    swaps = 0
    try:
        for step in range(400):
            t1, t2 = pt.choose(r)
            e1 = otp.choose_t1(values, len(values), mt)
            e2 = otp.choose_t2(LADDER, values, indices, 3, jump_type, e1, mt)
            assert (t1, t2) == (e1, e2), step
            s = pt.swap(r, t1, t2, like[step, t1 - 1], like[step, t2 - 1])
            es = otp.do_tempering(values, indices, t1, t2, like[step, t1 - 1], like[step, t2 - 1], mt)
            assert s == bool(es), step
            swaps += es
            assert list(pt.values) == values and list(pt.indices) == indices, step
            assert r.count() == draws[0]
    finally:
        r.close()
    assert pt.total == 400 and pt.accepted == swaps
    assert 0 < swaps < 400
    assert sorted(pt.values) == sorted(LADDER)


def test_tempered_acceptance_divides_the_ratio_by_the_temperature():
    settings = dict(ncell_min=4, ncell_max=40, kernel=0, datatype=2, sigdep=0, locate=0, xmin=0, xmax=1, ymin=0,
                    ymax=1, zmin=0, zmax=1, vpmin=0.5, vpmax=4.5, vsmin=0.3, vsmax=2.5, sigma_vp=0.1, sigma_vs=0.1,
                    sigma_vp2=0.1, sigma_vs2=0.1, pd=5.0, pd2=5.0, sigma_bn0=0, sigma_bn1=0, bn0_min=0, bn0_max=1,
                    bn1_min=0, bn1_max=1, sigma_sn0=0, sigma_sn1=0, sn0_min=0, sn0_max=1, sn1_min=0, sn1_max=1)
    ch = sampler.Chain(settings, 7, 4, np.full((40, 3), 0.5), np.full((40, 3), 1.0))
    rng = np.random.default_rng(3)
    try:
        for _ in range(2000):
            st = sampler.McmcStep(int(rng.integers(1, 7)), 1, 1, float(rng.normal()), float(rng.uniform(1e-6, 1)))
            new, old, t = rng.uniform(90, 110), rng.uniform(90, 110), float(rng.choice(LADDER))
            ratio = (-new + old) / t                       # mcmc_loc2.f90:881-886, 933-938, 979-981
            a = ratio
            if st.ptype == 1:
                a = st.prob - math.log(2.5 - 0.3) + ratio
            elif st.ptype == 2:
                a = st.prob + math.log(2.5 - 0.3) + ratio
            assert ch.accept_tempered(st, new, old, t) == (math.log(st.random) < min(0.0, a))
    finally:
        ch.close()
