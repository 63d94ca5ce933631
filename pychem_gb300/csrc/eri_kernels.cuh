// ERI kernel templates (one thread per shell quartet) -- included by the eri_g*.cu
// translation units, each of which instantiates a group of classes.
#pragma once
#include "common.cuh"
#include "pcg_internal.h"
#include "eri_gen.cuh"

struct PQd {
  double PAx, PAy, PAz, WPx, WPy, WPz, QCx, QCy, QCz, WQx, WQy, WQz, oo2z, oo2e, oo2ze, rz, re;
};
struct PQf {
  float PAx, PAy, PAz, WPx, WPy, WPz, QCx, QCy, QCz, WQx, WQy, WQz, oo2z, oo2e, oo2ze, rz, re;
};

template <class C>
__global__ void __launch_bounds__(128) k_eri(DevPairsExt pr, BoysTable bt, const int2* __restrict__ tasks,
                                             int ntask, double* __restrict__ store) {
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
      const double T = rho * fma(PQx, PQx, fma(PQy, PQy, PQz * PQz));
      double F[C::L + 1];
      boys_eval<C::L>(bt, T, F);
      const double pre = Kp * __ldg(pr.p.K + j) * rs;
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

// Single-precision variant for quartets whose Schwarz bound is below the mixed
// threshold; the pair data are rounded from the double arrays, results widened.
template <class C>
__global__ void __launch_bounds__(128) k_eri_f(DevPairsExt pr, BoysTable bt, const int2* __restrict__ tasks,
                                               int ntask, double* __restrict__ store) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntask) return;
  const int2 tk = tasks[t];
  const int i0 = __ldg(pr.p.ppoff + tk.x), i1 = i0 + __ldg(pr.p.npp_of + tk.x);
  const int j0 = __ldg(pr.p.ppoff + tk.y), j1 = j0 + __ldg(pr.p.npp_of + tk.y);
  float acc[C::NACC];
#pragma unroll
  for (int k = 0; k < C::NACC; ++k) acc[k] = 0.0f;
  if (pr.p.pf8) {
    // packed FP32 pair table: P - Q = (P - A) - (Q - C) + (A - C), the shell-centre
    // difference A - C formed once per quartet in double precision
    const float ACx = (float)((__ldg(pr.p.P + 3 * i0) - __ldg(pr.p.PA + 3 * i0)) -
                              (__ldg(pr.p.P + 3 * j0) - __ldg(pr.p.PA + 3 * j0)));
    const float ACy = (float)((__ldg(pr.p.P + 3 * i0 + 1) - __ldg(pr.p.PA + 3 * i0 + 1)) -
                              (__ldg(pr.p.P + 3 * j0 + 1) - __ldg(pr.p.PA + 3 * j0 + 1)));
    const float ACz = (float)((__ldg(pr.p.P + 3 * i0 + 2) - __ldg(pr.p.PA + 3 * i0 + 2)) -
                              (__ldg(pr.p.P + 3 * j0 + 2) - __ldg(pr.p.PA + 3 * j0 + 2)));
    for (int i = i0; i < i1; ++i) {
      const float4 a0 = __ldg(pr.p.pf8 + 2 * i), a1 = __ldg(pr.p.pf8 + 2 * i + 1);
      const float zeta = a0.x, Kp = a1.y;
      PQf q;
      q.PAx = a0.y; q.PAy = a0.z; q.PAz = a0.w;
      q.oo2z = a1.x;
      for (int j = j0; j < j1; ++j) {
        const float4 b0 = __ldg(pr.p.pf8 + 2 * j), b1 = __ldg(pr.p.pf8 + 2 * j + 1);
        const float eta = b0.x;
        const float PQx = (q.PAx - b0.y) + ACx;
        const float PQy = (q.PAy - b0.z) + ACy;
        const float PQz = (q.PAz - b0.w) + ACz;
        const float rs = rsqrtf(zeta + eta);
        const float izpe = rs * rs;
        const float rho = zeta * eta * izpe;
        const float T = rho * fmaf(PQx, PQx, fmaf(PQy, PQy, PQz * PQz));
        float F[C::L + 1];
        boys_eval_f<C::L>(bt, T, F);
        const float pre = Kp * b1.y * rs;
#pragma unroll
        for (int m = 0; m <= C::L; ++m) F[m] *= pre;
        const float wp = -eta * izpe, wq = zeta * izpe;
        q.WPx = wp * PQx; q.WPy = wp * PQy; q.WPz = wp * PQz;
        q.WQx = wq * PQx; q.WQy = wq * PQy; q.WQz = wq * PQz;
        q.QCx = b0.y; q.QCy = b0.z; q.QCz = b0.w;
        q.oo2e = b1.x;
        q.oo2ze = 0.5f * izpe;
        q.rz = eta * izpe;
        q.re = zeta * izpe;
        C::prim(q, F, acc);
      }
    }
  } else
  for (int i = i0; i < i1; ++i) {
    const double zd = __ldg(pr.p.zeta + i);
    const float zeta = (float)zd;
    const double Px = __ldg(pr.p.P + 3 * i), Py = __ldg(pr.p.P + 3 * i + 1), Pz = __ldg(pr.p.P + 3 * i + 2);
    const float Kp = __ldg(pr.p.Kf + i);
    PQf q;
    q.PAx = (float)__ldg(pr.p.PA + 3 * i);
    q.PAy = (float)__ldg(pr.p.PA + 3 * i + 1);
    q.PAz = (float)__ldg(pr.p.PA + 3 * i + 2);
    q.oo2z = (float)__ldg(pr.oo2z + i);
    for (int j = j0; j < j1; ++j) {
      const float eta = (float)__ldg(pr.p.zeta + j);
      const float PQx = (float)(Px - __ldg(pr.p.P + 3 * j));
      const float PQy = (float)(Py - __ldg(pr.p.P + 3 * j + 1));
      const float PQz = (float)(Pz - __ldg(pr.p.P + 3 * j + 2));
      const float rs = rsqrtf(zeta + eta);
      const float izpe = rs * rs;
      const float rho = zeta * eta * izpe;
      const float T = rho * fmaf(PQx, PQx, fmaf(PQy, PQy, PQz * PQz));
      float F[C::L + 1];
      boys_eval_f<C::L>(bt, T, F);
      const float pre = Kp * __ldg(pr.p.Kf + j) * rs;
#pragma unroll
      for (int m = 0; m <= C::L; ++m) F[m] *= pre;
      const float wp = -eta * izpe, wq = zeta * izpe;
      q.WPx = wp * PQx; q.WPy = wp * PQy; q.WPz = wp * PQz;
      q.WQx = wq * PQx; q.WQy = wq * PQy; q.WQz = wq * PQz;
      q.QCx = (float)__ldg(pr.p.PA + 3 * j);
      q.QCy = (float)__ldg(pr.p.PA + 3 * j + 1);
      q.QCz = (float)__ldg(pr.p.PA + 3 * j + 2);
      q.oo2e = (float)__ldg(pr.oo2z + j);
      q.oo2ze = 0.5f * izpe;
      q.rz = eta * izpe;
      q.re = zeta * izpe;
      C::prim(q, F, acc);
    }
  }
  const float ABx = (float)__ldg(pr.p.AB + 3 * tk.x), ABy = (float)__ldg(pr.p.AB + 3 * tk.x + 1),
              ABz = (float)__ldg(pr.p.AB + 3 * tk.x + 2);
  const float CDx = (float)__ldg(pr.p.AB + 3 * tk.y), CDy = (float)__ldg(pr.p.AB + 3 * tk.y + 1),
              CDz = (float)__ldg(pr.p.AB + 3 * tk.y + 2);
  C::finish(acc, ABx, ABy, ABz, CDx, CDy, CDz, [&](int k, float v) { store[(size_t)k * ntask + t] = (double)v; });
}

