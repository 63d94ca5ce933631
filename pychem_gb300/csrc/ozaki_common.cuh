// Device helpers of the Ozaki-scheme GEMMs (ozaki.cu, oz_tc.cu): the signed 7-bit
// digit split of an FP64 value against its vector's exponent, and the exact rounding
// of an int64 level sum times a power of two to FP64.  Integer operations only.
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

#ifndef OZ_BETA
#define OZ_BETA 7
#endif

__device__ __forceinline__ unsigned long long oz_absbits(double x) {
  return (unsigned long long)__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFull;
}

// The 63-bit fixed-point magnitude F = |x| 2^{63-e} of x for the exponent field emax
// of its vector's largest |x| (max |x| < 2^e, e = emax - 1022), biased for the signed
// digit split: G = F + B with B = sum_p 64 * 2^{63 - 7p} + 2^{62 - 7 NS}.  Then
// u_p = (G >> (63 - 7p)) & 127 (no mask for p = 1) gives the balanced base-128 digits
// d_p = u_p - 64 of F rounded to nearest at the last digit: the additions of 64 carry
// exactly as the signed-digit rebalancing would, d_1 in [0, 128], d_p in [-64, 63].
template <int NS>
__device__ __forceinline__ unsigned long long oz_biased(double x, int emax) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  const int e = emax ? emax - 1022 : 0;
  const int ex = (int)((u >> 52) & 0x7FF);
  unsigned long long F = 0;
  if (ex != 0 && emax != 0) {
    const unsigned long long mant = (u & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    const int sh = ex - 1012 - e;  // F = mant 2^sh < 2^63
    if (sh >= 0) F = mant << sh;
    else if (sh > -64) F = mant >> (-sh);
  }
  unsigned long long B = 1ull << (62 - OZ_BETA * NS);
#pragma unroll
  for (int p = 1; p <= NS; ++p) B += 64ull << (63 - OZ_BETA * p);
  return F + B;
}

template <int NS>
__device__ __forceinline__ int oz_digit(unsigned long long G, int p) {  // p = 1 .. NS
  return p == 1 ? (int)(G >> (63 - OZ_BETA)) - 64 : (int)((G >> (63 - OZ_BETA * p)) & 127ull) - 64;
}

// The NS signed digits of x for the exponent field emax of its vector's max:
// x = 2^e sum_p d_p 2^{-7p} + O(2^{e - 7 NS - 1}), |d_1| <= 128, |d_p| <= 64.
template <int NS>
__device__ __forceinline__ void oz_digits(double x, int emax, int* d) {
  const unsigned long long G = oz_biased<NS>(x, emax);
  const int neg = (int)((unsigned long long)__double_as_longlong(x) >> 63);
#pragma unroll
  for (int p = 1; p <= NS; ++p) {
    const int v = oz_digit<NS>(G, p);
    d[p - 1] = neg ? -v : v;
  }
}

// acc 2^e as a double, rounded to nearest even like an int64 -> FP64 conversion, built
// with integer operations only (64-bit conversions run on the FP64 pipe); results
// below the normal range are flushed to 0 (far under any tolerance here).
__device__ __forceinline__ double oz_ll_scaled(long long acc, int e) {
  if (acc == 0) return 0.0;
  const unsigned long long sign = acc < 0 ? 1ull : 0ull;
  unsigned long long mag = sign ? (unsigned long long)(-acc) : (unsigned long long)acc;
  int msb = 63 - __clzll((long long)mag);
  unsigned long long mant;
  if (msb <= 52) {
    mant = mag << (52 - msb);
  } else {
    const int sh = msb - 52;
    mant = mag >> sh;
    const unsigned long long rem = mag & ((1ull << sh) - 1ull), half = 1ull << (sh - 1);
    if (rem > half || (rem == half && (mant & 1ull))) ++mant;
    if (mant >> 53) { mant >>= 1; ++msb; }
  }
  const int ef = msb + 1023 + e;
  if (ef <= 0) return 0.0;
  return __longlong_as_double((long long)((sign << 63) | ((unsigned long long)ef << 52) | (mant & 0xFFFFFFFFFFFFFull)));
}

// The same digits for two values at once, packed as BF16 pairs: w[p-1] holds digit p of
// x0 (low half) and x1 (high half).  32-bit work only: the top 7 NS + 1 bits of
// |x| 2^{63-e} are one right shift of the 53-bit mantissa (the shift is at least
// 52 - 7 NS >= 3 because |x| < 2^e), the bias of oz_biased (in these units: 64 at
// every digit and 1 at the rounding bit) is a constant, a digit is one shift and mask,
// u - 64 becomes an exact float as (2^23 + u) - (2^23 + 64), and the signs are applied
// to the packed pair with one XOR.  Identical digits to oz_digits.
template <int NS>
__device__ __forceinline__ unsigned long long oz_top_biased(double x, int emax) {
  const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
  const int ex = (int)((hi >> 20) & 0x7FFu);
  const int e = emax ? emax - 1022 : 0;
  const int sft = (62 - OZ_BETA * NS) - (ex - 1012 - e);
  unsigned long long R = 0;
  if (ex != 0 && emax != 0 && sft < 53) {
    const unsigned mh = (hi & 0xFFFFFu) | 0x100000u;
    unsigned rl, rh;
    if (sft < 32) {
      rl = __funnelshift_r(lo, mh, sft);
      rh = mh >> sft;
    } else {
      rl = mh >> (sft - 32);
      rh = 0u;
    }
    R = ((unsigned long long)rh << 32) | rl;
  }
  unsigned long long B = 1ull;
#pragma unroll
  for (int p = 1; p <= NS; ++p) B += 64ull << (1 + OZ_BETA * (NS - p));
  return R + B;
}

__device__ __forceinline__ float oz_u7_to_float(unsigned u) {  // u - 64 for u in [0, 255], exact
  return __int_as_float(0x4B000000 | (int)u) - 8388672.0f;
}

template <int NS>
__device__ __forceinline__ void oz_digits_bf16x2(double x0, double x1, int emax, unsigned* w) {
  const unsigned long long G0 = oz_top_biased<NS>(x0, emax), G1 = oz_top_biased<NS>(x1, emax);
  const unsigned sg = ((unsigned)__double2hiint(x0) >> 31 ? 0x8000u : 0u) |
                      ((unsigned)__double2hiint(x1) >> 31 ? 0x80000000u : 0u);
#pragma unroll
  for (int p = 1; p <= NS; ++p) {
    const int b = 1 + OZ_BETA * (NS - p);
    const unsigned u0 = p == 1 ? (unsigned)(G0 >> b) : (unsigned)(G0 >> b) & 127u;
    const unsigned u1 = p == 1 ? (unsigned)(G1 >> b) : (unsigned)(G1 >> b) & 127u;
    __nv_bfloat162 b2 = __floats2bfloat162_rn(oz_u7_to_float(u0), oz_u7_to_float(u1));
    w[p - 1] = *(unsigned*)&b2 ^ sg;
  }
}
