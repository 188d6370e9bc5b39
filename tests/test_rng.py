"""CPU: the sampler's random number stream (the reference's mt19937 module,
src/mt19937.f90) through the C ABI; no GPU is needed.

Known answers: MT19937 seeded with init_genrand(5489) is the generator the
C++ standard names std::mt19937, whose first output is 3499211612 and whose
10000th output is 4123659995 ([rand.predef]).
"""
import ctypes
import math

import pytest

from mctomo_gb300 import lib


@pytest.fixture()
def rng():
    L = lib()
    h = ctypes.c_void_p()
    assert L.mct_rng_create(5489, ctypes.byref(h)) == 0
    yield L, h
    L.mct_rng_destroy(h)


def test_mt19937_known_answers(rng):
    L, h = rng
    assert L.mct_rng_u32(h) == 3499211612
    for _ in range(9998):
        L.mct_rng_u32(h)
    assert L.mct_rng_u32(h) == 4123659995
    assert L.mct_rng_count(h) == 10000


def test_unirand_and_gasdev_follow_grnd(rng):
    L, h = rng
    g = ctypes.c_void_p()
    assert L.mct_rng_create(5489, ctypes.byref(g)) == 0
    try:
        # unirand = grnd = u / (2^32 - 1) of the same stream
        for _ in range(1000):
            assert L.mct_rng_unirand(h) == L.mct_rng_u32(g) / 4294967295.0
        # gasdev: polar method on pairs of grnd draws, rejection included
        for _ in range(1000):
            while True:
                v1 = 2 * (L.mct_rng_u32(g) / 4294967295.0) - 1
                v2 = 2 * (L.mct_rng_u32(g) / 4294967295.0) - 1
                r = v1 * v1 + v2 * v2
                if r < 1 and r != 0:
                    break
            assert L.mct_rng_gasdev(h) == v2 * math.sqrt(-2 * math.log(r) / r)
        assert L.mct_rng_count(h) == L.mct_rng_count(g)
    finally:
        L.mct_rng_destroy(g)


def test_reseeding_restarts_the_stream(rng):
    L, h = rng
    a = [L.mct_rng_unirand(h) for _ in range(5)]
    assert L.mct_rng_seed(h, 5489) == 0
    assert L.mct_rng_count(h) == 0
    assert [L.mct_rng_unirand(h) for _ in range(5)] == a
