// Spherical Bessel functions for the j0(S r12) electron-scattering operator
// (Methods/c_ints/spherical_bessel_j.c), shared by the scattering ERI kernels
// (eri_scat.cuh) and the drop-in fundamentals (compat.cu).
#pragma once
#include <cuda_runtime.h>

// sin x and cos x for 10 <= x <~ 1e6 without a library call (a call's out-of-line
// slow path makes the large classes spill their accumulators): Cody-Waite reduction
// x = k pi/2 + r with pi/2 split into three parts (the first two with 33 significant
// bits, so k times either is exact for k < 2^20; computed from pi by Machin's
// formula), |r| <= pi/4, then the Taylor series of sin r to r^21 and of cos r to r^20
// (remainders below 1e-19).  Absolute error about 1e-16 over that range.
__device__ __forceinline__ void sincos_reduced(double x, double* sn, double* cs) {
  const double k = rint(x * 0.6366197723675814);
  double r = fma(-k, 1.5707963267341256, x);
  r = fma(-k, 6.077100506303966e-11, r);
  r = fma(-k, 2.0222662487959506e-21, r);
  const double r2 = r * r;
  double s = 1.0 / 51090942171709440000.0;                  // 1/21!
  s = fma(s, -r2, 1.0 / 121645100408832000.0);              // 1/19!
  s = fma(s, -r2, 1.0 / 355687428096000.0);                 // 1/17!
  s = fma(s, -r2, 1.0 / 1307674368000.0);                   // 1/15!
  s = fma(s, -r2, 1.0 / 6227020800.0);                      // 1/13!
  s = fma(s, -r2, 1.0 / 39916800.0);                        // 1/11!
  s = fma(s, -r2, 1.0 / 362880.0);                          // 1/9!
  s = fma(s, -r2, 1.0 / 5040.0);                            // 1/7!
  s = fma(s, -r2, 1.0 / 120.0);                             // 1/5!
  s = fma(s, -r2, 1.0 / 6.0);                               // 1/3!
  s = fma(s, -r2, 1.0);
  s *= r;
  double c = 1.0 / 2432902008176640000.0;                   // 1/20!
  c = fma(c, -r2, 1.0 / 6402373705728000.0);                // 1/18!
  c = fma(c, -r2, 1.0 / 20922789888000.0);                  // 1/16!
  c = fma(c, -r2, 1.0 / 87178291200.0);                     // 1/14!
  c = fma(c, -r2, 1.0 / 479001600.0);                       // 1/12!
  c = fma(c, -r2, 1.0 / 3628800.0);                         // 1/10!
  c = fma(c, -r2, 1.0 / 40320.0);                           // 1/8!
  c = fma(c, -r2, 1.0 / 720.0);                             // 1/6!
  c = fma(c, -r2, 1.0 / 24.0);                              // 1/4!
  c = fma(c, -r2, 0.5);                                     // 1/2!
  c = fma(c, -r2, 1.0);
  const int q = ((int)k) & 3;
  *sn = q == 0 ? s : (q == 1 ? c : (q == 2 ? -s : -c));
  *cs = q == 0 ? c : (q == 1 ? -s : (q == 2 ? -c : s));
}

// z^-m j_m(z), m = 0..L, by the regimes of spherical_bessel_j.c:5-81: the power series
// about 0 below z = 10 (1, 3, 6 or 20 terms by the size of z), the two-term asymptotic
// form above 100, upward recursion from j0 and j1 between; magnitudes below 1e-16 are
// set to 0.
template <int L>
__device__ __forceinline__ void sph_bessel_scaled(double z, double* j) {
  if (z < 10.0) {
    const int kmax = z < 1e-3 ? 1 : (z < 1e-1 ? 3 : (z < 1.0 ? 6 : 20));
    const double mz2 = -z * z;
    double df = 1.0;
#pragma unroll
    for (int m = 0; m <= L; ++m) {
      df *= (double)(2 * m + 1);
      // term_k = (-z^2)^k / (2^k k! (2m+3)(2m+5)...(2m+2k+1))
      double term = 1.0, sum = 1.0;
      for (int k = 1; k <= kmax; ++k) {
        term *= mz2 / ((2.0 * k) * (double)(2 * m + 2 * k + 1));
        sum += term;
      }
      j[m] = sum / df;
    }
  } else {
    double sz, cz;
    sincos_reduced(z, &sz, &cz);
    const double zi = 1.0 / z;
    if (z > 100.0) {
      // j_m(z) ~ sin(z - m pi/2)/z + m(m+1)/2 cos(z - m pi/2)/z^2
      double zm = 1.0;
      j[0] = sz * zi;
#pragma unroll
      for (int m = 1; m <= L; ++m) {
        zm *= zi;
        const int q = m & 3;   // sin and cos of z - m pi/2 by quarter turns
        const double s = q == 0 ? sz : (q == 1 ? -cz : (q == 2 ? -sz : cz));
        const double c = q == 0 ? cz : (q == 1 ? sz : (q == 2 ? -cz : -sz));
        j[m] = zm * (zi * s + (double)(m * (m + 1) / 2) * zi * zi * c);
      }
    } else {
      double r0 = sz * zi, r1 = (sz - z * cz) * zi * zi, zm = zi;
      j[0] = r0;
      if (L > 0) j[1] = r1 * zi;
#pragma unroll
      for (int m = 2; m <= L; ++m) {
        const double r2 = (2 * m - 1) * r1 * zi - r0;   // j_m from j_{m-1}, j_{m-2}
        zm *= zi;                                         // z^-m
        j[m] = r2 * zm;
        r0 = r1;
        r1 = r2;
      }
    }
  }
#pragma unroll
  for (int m = 0; m <= L; ++m)
    if (fabs(j[m]) < 1e-16) j[m] = 0.0;
}

// Runtime order 0..8 (the drop-in layer's l_max is a call argument).
__device__ __forceinline__ void sph_bessel_scaled_rt(int lmax, double z, double* j) {
  switch (lmax) {
    case 0: sph_bessel_scaled<0>(z, j); break;
    case 1: sph_bessel_scaled<1>(z, j); break;
    case 2: sph_bessel_scaled<2>(z, j); break;
    case 3: sph_bessel_scaled<3>(z, j); break;
    case 4: sph_bessel_scaled<4>(z, j); break;
    case 5: sph_bessel_scaled<5>(z, j); break;
    case 6: sph_bessel_scaled<6>(z, j); break;
    case 7: sph_bessel_scaled<7>(z, j); break;
    default: sph_bessel_scaled<8>(z, j); break;
  }
}
