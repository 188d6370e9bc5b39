// Correctly rounded FP64 square root computed on the integer and FP32 pipes.
//
// GB300 issues two FP64 lanes per cycle per SM, and a dependent FP64
// operation takes about 77 cycles, so an FP64 square root (a chain of
// dependent FP64 operations) is both long-latency and a large share of the
// FP64 pipe in the travel-time updates. This version produces the same bits
// (IEEE round to nearest even) for every input, but does the work with
// 32/64-bit integer arithmetic and a few FP32 estimates:
//
//   x = M * 2^e with M in [2^52, 2^53); after making e even (M2 = M or 2M),
//   sqrt(x) = sqrt(M2 * 2^52) * 2^(e/2 - 26), and the result's significand is
//   Y = RN(sqrt(N)), N = M2 * 2^52 < 2^106.
//
//   1. S1 = floor(sqrt(M2)) (27 bits) from an FP32 reciprocal-square-root
//      estimate, one Newton correction on the exact integer remainder
//      M2 - S^2, and an exact fix-up, so that R1 = M2 - S1^2 is in [0, 2 S1].
//   2. Y = S1 * 2^26 + T with T ~ 2^25 R1 / S1 (FP32), then one Newton
//      correction on the exact remainder N - Y^2. That remainder is below
//      2^59 in magnitude, so it is computed exactly modulo 2^64 from
//      N - Y^2 = R1 2^52 - S1 T 2^27 - T^2.
//   3. Rounding from the exact remainder: Y = RN(sqrt(N)) exactly when
//      -Y < N - Y^2 <= Y (sqrt(N) is never a half-integer), otherwise Y moves
//      by one.
//
// This is the square root with remainder of R. Brent and P. Zimmermann,
// "Modern Computer Arithmetic" (Cambridge University Press, 2010), section
// 1.5.1 (Newton steps on integer approximations, the remainder deciding the
// last unit), followed by the round-to-nearest rule on the remainder. Zero,
// subnormal, negative, infinite and NaN inputs take the library square root.
// The result is checked bit for bit against CUDA's sqrt by
// mct_debug_exact_sqrt_check.
#pragma once
#include <cuda_runtime.h>

__device__ __forceinline__ double exact_sqrt_rn(double x) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
  const unsigned E = (unsigned)(bits >> 52);   // sign bit included: positive inputs have E < 2048
  if (E - 1u >= 2046u) {                        // zero, subnormal, negative, infinite or NaN
    return sqrt(x);
  }
  const unsigned long long M = (bits & 0xFFFFFFFFFFFFFull) | (1ull << 52);
  const int e = (int)E - 1075;                  // x = M * 2^e
  const int odd = e & 1;
  const unsigned long long M2 = M << odd;       // [2^52, 2^54)
  const int eh = (e - odd) / 2;                 // exact: e - odd is even
  // 1. S1 = floor(sqrt(M2)), R1 = M2 - S1^2
  const float fM = __uint2float_rn((unsigned)(M2 >> 22)) * 4194304.0f;   // 2^22
  const float r = rsqrtf(fM);
  unsigned S = (unsigned)__float2uint_rn(fM * r);
  long long R = (long long)(M2 - (unsigned long long)S * S);
  S = (unsigned)((int)S + __float2int_rn(__int2float_rn((int)(R >> 8)) * (128.0f * r)));
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    R = (long long)(M2 - (unsigned long long)S * S);
    if (R < 0) S -= 1u;
    else if (R > 2ll * S) S += 1u;
  }
  const unsigned long long S1 = S;
  const unsigned long long R1 = M2 - S1 * S1;   // in [0, 2 S1]
  // 2. T ~ sqrt(N) - S1 2^26, one Newton correction on the exact remainder
  const float fS = __uint2float_rn(S);
  long long T = __float2int_rn(__uint2float_rn((unsigned)R1) * (33554432.0f / fS));   // 2^25
  auto rem = [&](long long t) {
    const unsigned long long ut = (unsigned long long)t;
    return (long long)((R1 << 52) - ((S1 * ut) << 27) - ut * ut);
  };
  T += __float2int_rn(__int2float_rn((int)(rem(T) >> 28)) * (2.0f / fS));
  // 3. round to nearest from the exact remainder
  long long Y = (long long)(S1 << 26) + T;
  const long long Rm = rem(T);
  if (Rm > Y) Y += 1;
  else if (Rm <= -Y) Y -= 1;
  const unsigned long long out = ((unsigned long long)(eh + 1049) << 52) | ((unsigned long long)Y & 0xFFFFFFFFFFFFFull);
  return __longlong_as_double((long long)out);
}
