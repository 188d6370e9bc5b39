"""ORACLE (test infrastructure only): parallel tempering of the reference's
mcmc_pt restated in plain Python, with its own MT19937.

* Mt: MT19937 seeded by init_genrand (Matsumoto and Nishimura, ACM TOMACS
  8(1), 1998; src/mt19937.f90:96-115) and the reference's grnd = u /
  (2^32 - 1) (:117-172), unirand = grnd (:224-236).
* choose_t1 (src/mcmc_loc2.f90:2148-2169), choose_t2 (:2171-2236) and
  do_tempering (:2240-2280) on 1-based chain numbers, with the ladder
  arrays temperature_values0 / temperature_indices0 (indices0(i) = i,
  run_time_info.f90:189) and the chains' current temperature_values /
  temperature_indices as Python lists (index 0 is chain 1).
* EPS is mcmc_loc2.f90:51's eps = 1e-8, a REAL*4 literal widened to REAL*8.
"""
import math
import struct

EPS = struct.unpack("f", struct.pack("f", 1e-8))[0]


class Mt:
    def __init__(self, seed):
        self.mt = [0] * 624
        self.mt[0] = seed & 0xFFFFFFFF
        for i in range(1, 624):
            prev = self.mt[i - 1]
            self.mt[i] = (1812433253 * (prev ^ (prev >> 30)) + i) & 0xFFFFFFFF
        self.mti = 624

    def u32(self):
        if self.mti >= 624:
            for k in range(624):
                y = (self.mt[k] & 0x80000000) | (self.mt[(k + 1) % 624] & 0x7FFFFFFF)
                self.mt[k] = self.mt[(k + 397) % 624] ^ (y >> 1) ^ (0x9908B0DF if y & 1 else 0)
            self.mti = 0
        y = self.mt[self.mti]
        self.mti += 1
        y ^= y >> 11
        y ^= (y << 7) & 0x9D2C5680
        y ^= (y << 15) & 0xEFC60000
        y ^= y >> 18
        return y

    def unirand(self):
        return self.u32() / 4294967295.0


def _ceil_index(u, n):
    i = math.ceil(u * n)
    return 1 if i == 0 else i


def choose_t1(values, n, mt):
    t1 = 0
    while not (1 <= t1 <= n):
        t1 = _ceil_index(mt.unirand(), n)
    return t1


def choose_t2(values0, values, indices, number_of_1s, jump_type, t1, mt):
    n = len(values)
    t1v, t1i = values[t1 - 1], indices[t1 - 1]
    if jump_type == 0:
        t2, t2v = 0, None
        while not (1 <= t2 <= n) or (t2v is not None and abs(t1v - t2v) < EPS):
            t2 = _ceil_index(mt.unirand(), n)
            t2v = values[t2 - 1]
        return t2
    if abs(t1v - 1.0) < EPS:
        k = number_of_1s + 1
    elif abs(t1v - values0[n - 1]) < EPS:
        k = n - 1
    elif jump_type == 1:
        k = t1i + (-1 if mt.unirand() < 0.5 else 1)
    else:
        best, k = None, 0
        for q in range(1, n + 1):
            d = abs(values0[q - 1] - t1v)
            if d > EPS and (best is None or d < best):
                best, k = d, q
        if k == 1:
            k = _ceil_index(mt.unirand(), number_of_1s)
    t2_index = k
    dist = [abs(i - t2_index) for i in indices]
    return dist.index(min(dist)) + 1


def do_tempering(values, indices, t1, t2, like1, like2, mt):
    """Returns 1 when the two chains swap temperatures (in place), else 0."""
    t1v, t2v = values[t1 - 1], values[t2 - 1]
    alpha = min(0.0, -(like1 / t2v) + like2 / t2v - like2 / t1v + like1 / t1v)
    u = mt.unirand()
    if (math.log(u) if u > 0 else -math.inf) <= alpha:
        values[t1 - 1], values[t2 - 1] = values[t2 - 1], values[t1 - 1]
        indices[t1 - 1], indices[t2 - 1] = indices[t2 - 1], indices[t1 - 1]
        return 1
    return 0
