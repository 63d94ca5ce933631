// Electron-scattering integrals (ab|j0(S r12)|cd) -- the operator of
// Methods/properties.py:20-23, integrals of Methods/c_ints/two_electron_scattering.c
// and spherical_bessel_j.c.  One thread per shell quartet, the generated VRR/HRR of
// the Coulomb kernels; only the fundamentals differ.  Included by eri_s*.cu.
#pragma once
#include "eri_kernels.cuh"
#include "scat_fund.cuh"

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
