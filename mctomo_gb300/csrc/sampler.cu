// Host side of the reversible-jump sampler: the reference's random number
// stream (src/mt19937.f90), so that a C or Fortran host can drive the GPU
// likelihood with the reference's own sequence of random draws. Host code
// only (no kernels).
//
// MT19937 (M. Matsumoto and T. Nishimura, "Mersenne Twister: a
// 623-dimensionally equidistributed uniform pseudo-random number generator",
// ACM TOMACS 8(1), 1998) seeded by init_genrand's recursion
// (src/mt19937.f90:96-115), with the reference's real conversion
// grnd = u / (2^32 - 1) of the 32-bit output u (:117-172), unirand = grnd
// (:224-236) and gasdev, the polar Box-Muller method on two grnd draws
// (:200-222). Each generator counts its draws as RTI%randcount does.
#include "mct_common.cuh"
#include <cmath>
#include <new>

struct mct_rng {
  unsigned mt[624];
  int mti;
  long long count;   // draws so far (RTI%randcount)
};

namespace {

constexpr int kN = 624, kM = 397;
constexpr unsigned kMatrixA = 0x9908B0DFu, kUpper = 0x80000000u, kLower = 0x7FFFFFFFu;

void init_genrand(mct_rng *r, unsigned seed) {
  r->mt[0] = seed;
  for (int i = 1; i < kN; ++i) {
    const unsigned prev = r->mt[i - 1];
    r->mt[i] = 1812433253u * (prev ^ (prev >> 30)) + (unsigned)i;
  }
  r->mti = kN;
}

unsigned next_u32(mct_rng *r) {
  if (r->mti >= kN) {
    for (int k = 0; k < kN; ++k) {
      const unsigned y = (r->mt[k] & kUpper) | (r->mt[(k + 1) % kN] & kLower);
      r->mt[k] = r->mt[(k + kM) % kN] ^ (y >> 1) ^ ((y & 1u) ? kMatrixA : 0u);
    }
    r->mti = 0;
  }
  unsigned y = r->mt[r->mti++];
  y ^= y >> 11;
  y ^= (y << 7) & 0x9D2C5680u;
  y ^= (y << 15) & 0xEFC60000u;
  y ^= y >> 18;
  return y;
}

// grnd: the unsigned 32-bit output over 2^32 - 1, in double
double grnd(mct_rng *r) { return (double)next_u32(r) / (4294967296.0 - 1.0); }

}  // namespace

extern "C" {

int mct_rng_create(unsigned seed, mct_rng **out) {
  if (!out) return MCT_ERR_ARG;
  mct_rng *r = new (std::nothrow) mct_rng;
  if (!r) return MCT_ERR_NOMEM;
  init_genrand(r, seed);
  r->count = 0;
  *out = r;
  return MCT_OK;
}

void mct_rng_destroy(mct_rng *r) { delete r; }

int mct_rng_seed(mct_rng *r, unsigned seed) {
  if (!r) return MCT_ERR_ARG;
  init_genrand(r, seed);
  r->count = 0;
  return MCT_OK;
}

double mct_rng_unirand(mct_rng *r) {
  const double v = grnd(r);
  ++r->count;
  return v;
}

double mct_rng_gasdev(mct_rng *r) {
  for (;;) {
    const double v1 = 2 * grnd(r) - 1;
    ++r->count;
    const double v2 = 2 * grnd(r) - 1;
    ++r->count;
    const double rr = v1 * v1 + v2 * v2;
    if (rr >= 1 || rr == 0) continue;
    const double fac = std::sqrt(-2 * std::log(rr) / rr);
    return v2 * fac;
  }
}

unsigned mct_rng_u32(mct_rng *r) {
  ++r->count;
  return next_u32(r);
}

long long mct_rng_count(const mct_rng *r) { return r ? r->count : -1; }

}  // extern "C"
