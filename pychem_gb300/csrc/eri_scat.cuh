// Electron-scattering integrals (ab|j0(S r12)|cd) -- the operator of
// Methods/properties.py:20-23, integrals of Methods/c_ints/two_electron_scattering.c
// and spherical_bessel_j.c.  One thread per shell quartet, the generated VRR/HRR of
// the Coulomb kernels; only the fundamentals differ.  Included by eri_s*.cu.
#pragma once
#include "eri_kernels.cuh"

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

// Fundamentals of j0(S r12) in the Obara-Saika form used by the generated VRR:
// (-d/dT)^m of exp(-S^2/(4 rho)) j0(S R) at T = rho R^2, i.e.
// exp(-S^2/(4 rho)) (S^2/(2 rho))^m z^-m j_m(z) with z = S R; the S = 0 and R = 0
// cases as two_electron_scattering.c:47-66.
template <int L>
__device__ __forceinline__ void scat_eval(double S, double rho, double R2, double* F) {
  if (S < 1e-14) {
    F[0] = 1.0;
#pragma unroll
    for (int m = 1; m <= L; ++m) F[m] = 0.0;
    return;
  }
  const double eS = exp(-0.25 * S * S / rho), step = S * S / (2.0 * rho);
  if (R2 < 1e-14) {
    double df = 1.0, sp = eS;
#pragma unroll
    for (int m = 0; m <= L; ++m) {
      df *= (double)(2 * m + 1);
      F[m] = sp / df;
      sp *= step;
    }
  } else {
    sph_bessel_scaled<L>(S * sqrt(R2), F);
    double sp = eS;
#pragma unroll
    for (int m = 0; m <= L; ++m) {
      F[m] *= sp;
      sp *= step;
    }
  }
}

// The Coulomb kernel k_eri with the scattering fundamentals; the prefactor turns the
// pair factors K_P K_Q (which carry 2 pi^{5/2}/(zeta eta) for 1/r12) into the overlap
// product U_P U_Q: times sqrt(pi) / (2 sqrt(zeta eta)).
template <class C>
__global__ void __launch_bounds__(128) k_eri_s(DevPairsExt pr, const int2* __restrict__ tasks, int ntask, double S,
                                               double* __restrict__ store) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntask) return;
  const int2 tk = tasks[t];
  const int i0 = __ldg(pr.p.ppoff + tk.x), i1 = i0 + __ldg(pr.p.npp_of + tk.x);
  const int j0 = __ldg(pr.p.ppoff + tk.y), j1 = j0 + __ldg(pr.p.npp_of + tk.y);
  double acc[C::NACC];
#pragma unroll
  for (int k = 0; k < C::NACC; ++k) acc[k] = 0.0;
  for (int i = i0; i < i1; ++i) {
    const double zeta = __ldg(pr.p.zeta + i);
    const double Px = __ldg(pr.p.P + 3 * i), Py = __ldg(pr.p.P + 3 * i + 1), Pz = __ldg(pr.p.P + 3 * i + 2);
    const double Kp = __ldg(pr.p.K + i);
    PQd q;
    q.PAx = __ldg(pr.p.PA + 3 * i);
    q.PAy = __ldg(pr.p.PA + 3 * i + 1);
    q.PAz = __ldg(pr.p.PA + 3 * i + 2);
    q.oo2z = __ldg(pr.oo2z + i);
    for (int j = j0; j < j1; ++j) {
      const double eta = __ldg(pr.p.zeta + j);
      const double PQx = Px - __ldg(pr.p.P + 3 * j);
      const double PQy = Py - __ldg(pr.p.P + 3 * j + 1);
      const double PQz = Pz - __ldg(pr.p.P + 3 * j + 2);
      const double rs = nr_rsqrt(zeta + eta);
      const double izpe = rs * rs;
      const double rho = zeta * eta * izpe;
      double F[C::L + 1];
      scat_eval<C::L>(S, rho, fma(PQx, PQx, fma(PQy, PQy, PQz * PQz)), F);
      const double pre = Kp * __ldg(pr.p.K + j) * 0.88622692545275801365 * nr_rsqrt(zeta * eta);
#pragma unroll
      for (int m = 0; m <= C::L; ++m) F[m] *= pre;
      const double wp = -eta * izpe, wq = zeta * izpe;
      q.WPx = wp * PQx; q.WPy = wp * PQy; q.WPz = wp * PQz;
      q.WQx = wq * PQx; q.WQy = wq * PQy; q.WQz = wq * PQz;
      q.QCx = __ldg(pr.p.PA + 3 * j);
      q.QCy = __ldg(pr.p.PA + 3 * j + 1);
      q.QCz = __ldg(pr.p.PA + 3 * j + 2);
      q.oo2e = __ldg(pr.oo2z + j);
      q.oo2ze = 0.5 * izpe;
      q.rz = eta * izpe;
      q.re = zeta * izpe;
      C::prim(q, F, acc);
    }
  }
  const double ABx = __ldg(pr.p.AB + 3 * tk.x), ABy = __ldg(pr.p.AB + 3 * tk.x + 1), ABz = __ldg(pr.p.AB + 3 * tk.x + 2);
  const double CDx = __ldg(pr.p.AB + 3 * tk.y), CDy = __ldg(pr.p.AB + 3 * tk.y + 1), CDz = __ldg(pr.p.AB + 3 * tk.y + 2);
  C::finish(acc, ABx, ABy, ABz, CDx, CDy, CDz, [&](int k, double v) { store[(size_t)k * ntask + t] = v; });
}
