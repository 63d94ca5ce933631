// Shared device-side definitions for the pychem_gb300 integral/SCF library.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define PCG_MAXL 2               // shells up to d
#define PCG_MAXLT (4 * PCG_MAXL) // highest Boys order for an ERI class
#define PCG_MAXPRIM 16

// status codes of the C ABI (PCG_OK, PCG_ERR_*)
#include "../../include/pychem_gb300.h"

#define PCG_CUDA(call)                                      \
  do {                                                      \
    cudaError_t _e = (call);                                \
    if (_e != cudaSuccess) { pcg_set_cuda_error(_e, #call); \
      return PCG_ERR_CUDA; }                                \
  } while (0)

void pcg_set_cuda_error(cudaError_t e, const char* what);
void pcg_set_error(const char* msg);

// ----------------------------------------------------------------------------------
// Boys function F_m(T).  Grid T_p = p / 16 for T < BOYS_TMAX; per grid point the
// rows c[m][k] = F_{m+k}(T_p) / k! (k < BOYS_K) and exp(-T_p).  F_m(T) is the Taylor
// series about the nearest grid point (|dT| <= 1/32), truncation < 2e-17 relative for
// BOYS_K = 8.  Lower orders come from the downward recursion
//   F_{m-1} = (2T F_m + exp(-T)) / (2m - 1),
// exp(-T) from the same grid.  Beyond BOYS_TMAX: F_0 = sqrt(pi/T)/2 and the upward
// recursion F_{m+1} = (2m+1) F_m / (2T) (exp(-T) < 1e-20 there).
// ----------------------------------------------------------------------------------
#define BOYS_INV_H 16
#define BOYS_TMAX 48.0
#define BOYS_NP (48 * BOYS_INV_H + 1)
#define BOYS_K 8
#define BOYS_M (PCG_MAXLT + 1)
#define BOYS_KF 5  // terms for the single-precision variant

struct BoysTable {
  const double* c;    // [BOYS_NP][BOYS_M][BOYS_K]
  const double* ex;   // [BOYS_NP]
  const float* cf;    // [BOYS_NP][BOYS_M][BOYS_KF]
  const float* exf;   // [BOYS_NP]
};

// Reciprocal square root by Newton-Raphson refinement of the single-precision
// estimate: y <- y (3 - x y^2) / 2, quadratic convergence; two steps reach double
// precision from rsqrtf's ~2^-23 relative error.
__device__ __forceinline__ double nr_rsqrt(double x) {
  double y = (double)rsqrtf((float)x);
  double h = 0.5 * x;
  y = y * fma(-h * y, y, 1.5);
  y = y * fma(-h * y, y, 1.5);
  return y;
}

// Reciprocal by Newton-Raphson: y <- y (2 - x y), two steps from the float estimate.
__device__ __forceinline__ double nr_rcp(double x) {
  double y = (double)(1.0f / (float)x);
  double e = fma(-x, y, 1.0);
  y = fma(y, e, y);
  e = fma(-x, y, 1.0);
  y = fma(y, e, y);
  return y;
}

template <int L>
__device__ __forceinline__ void boys_eval(const BoysTable& bt, double T, double* F) {
  if (T < BOYS_TMAX) {
    // nearest grid point without conversions: adding 1.5 * 2^52 rounds T * 16 to an
    // integer held in the low mantissa bits
    const double r = fma(T, (double)BOYS_INV_H, 6755399441055744.0);
    const int p = __double2loint(r);
    const double d = (r - 6755399441055744.0) * (1.0 / BOYS_INV_H) - T;  // -(T - T_p)
    const double* row = bt.c + ((size_t)p * BOYS_M + L) * BOYS_K;
    double f = __ldg(row + BOYS_K - 1);
#pragma unroll
    for (int k = BOYS_K - 2; k >= 0; --k) f = fma(f, d, __ldg(row + k));
    F[L] = f;
    if (L > 0) {
      // exp(-T) = exp(-T_p) * sum_k d^k / k!
      double e = 1.0 / 5040.0;
      e = fma(e, d, 1.0 / 720.0);
      e = fma(e, d, 1.0 / 120.0);
      e = fma(e, d, 1.0 / 24.0);
      e = fma(e, d, 1.0 / 6.0);
      e = fma(e, d, 0.5);
      e = fma(e, d, 1.0);
      e = fma(e, d, 1.0);
      e *= __ldg(bt.ex + p);
      const double t2 = 2.0 * T;
#pragma unroll
      for (int m = L; m > 0; --m) F[m - 1] = fma(t2, F[m], e) * (1.0 / (2 * m - 1));
    }
  } else {
    const double rs = nr_rsqrt(T);
    F[0] = 0.88622692545275801365 * rs;  // sqrt(pi)/2
    if (L > 0) {
      const double h = 0.5 * rs * rs;      // 1 / (2T)
#pragma unroll
      for (int m = 0; m < L; ++m) F[m + 1] = F[m] * ((2 * m + 1) * h);
    }
  }
}

template <int L>
__device__ __forceinline__ void boys_eval_f(const BoysTable& bt, float T, float* F) {
  if (T < (float)BOYS_TMAX) {
    const int p = __float2int_rn(T * BOYS_INV_H);
    const float d = (float)p * (1.0f / BOYS_INV_H) - T;
    const float* row = bt.cf + ((size_t)p * BOYS_M + L) * BOYS_KF;
    float f = __ldg(row + BOYS_KF - 1);
#pragma unroll
    for (int k = BOYS_KF - 2; k >= 0; --k) f = fmaf(f, d, __ldg(row + k));
    F[L] = f;
    if (L > 0) {
      float e = 1.0f / 24.0f;
      e = fmaf(e, d, 1.0f / 6.0f);
      e = fmaf(e, d, 0.5f);
      e = fmaf(e, d, 1.0f);
      e = fmaf(e, d, 1.0f);
      e *= __ldg(bt.exf + p);
      const float t2 = 2.0f * T;
#pragma unroll
      for (int m = L; m > 0; --m) F[m - 1] = fmaf(t2, F[m], e) * (1.0f / (2 * m - 1));
    }
  } else {
    const float rs = rsqrtf(T);
    F[0] = 0.88622692545275801365f * rs;
    if (L > 0) {
      const float h = 0.5f * rs * rs;
#pragma unroll
      for (int m = 0; m < L; ++m) F[m + 1] = F[m] * ((2 * m + 1) * h);
    }
  }
}

// runtime-L dispatch used by the one-electron kernels and fine-grained entry points
__device__ __forceinline__ void boys_eval_rt(const BoysTable& bt, int L, double T, double* F) {
  switch (L) {
    case 0: boys_eval<0>(bt, T, F); break;
    case 1: boys_eval<1>(bt, T, F); break;
    case 2: boys_eval<2>(bt, T, F); break;
    case 3: boys_eval<3>(bt, T, F); break;
    case 4: boys_eval<4>(bt, T, F); break;
    case 5: boys_eval<5>(bt, T, F); break;
    case 6: boys_eval<6>(bt, T, F); break;
    case 7: boys_eval<7>(bt, T, F); break;
    default: boys_eval<8>(bt, T, F); break;
  }
}

// ----------------------------------------------------------------------------------
// Basis and pair data in HBM (structure of arrays).
//   shells:      l, nprim, first primitive, first AO (spherical), atom, centre
//   primitives:  exponent, contraction coefficient times (2a)^{(l+1.5)/2} times the
//                normalisation of the pure-axis Cartesian component
//   shell pairs: oriented A = higher l; primitive pairs of pair p are
//                [ppoff[p], ppoff[p] + npp[p]), row-major over (primA, primB)
//   prim pairs:  zeta, P, P - A, and K = cc_a cc_b (2/sqrt(pi))^{1/2} U sqrt(zeta)
//                with U = (pi/zeta)^{3/2} exp(-ab/zeta |A-B|^2), so that
//                [00|00]^(m) = K_P K_Q F_m(T) / sqrt(zeta + eta)
// ----------------------------------------------------------------------------------
struct DevBasis {
  int nshell, nprim, natom, nbf;
  const int* sh_l;
  const int* sh_nprim;
  const int* sh_prim;
  const int* sh_ao;
  const int* sh_atom;
  const double* sh_xyz;      // [nshell][3]
  const double* pr_exp;
  const double* pr_cc;
  const double* at_xyz;      // [natom][3]
  const double* at_z;
  // matrix layout: element (p, q) of the shell's molecule lives at
  //   blk(shell) + p * ld + q   (p, q local AO indices); a single molecule has
  //   blk = 0, ld = nbf.  Nuclear attraction runs over the molecule's atoms only.
  int ld;
  const long long* sh_blk;   // nullptr: 0 for every shell
  const int* sh_at0;         // nullptr: atoms [0, natom)
  const int* sh_nat;
};

__device__ __forceinline__ long long dev_blk(const DevBasis& b, int sh) {
  return b.sh_blk ? __ldg(b.sh_blk + sh) : 0ll;
}

struct DevPairs {
  int npair, npp;
  const int* A;       // shell index, l_A >= l_B
  const int* B;
  const int* ppoff;
  const int* npp_of;
  const double* AB;   // [npair][3] = A - B
  // primitive-pair SoA
  const double* zeta;
  const double* P;    // [npp][3]
  const double* PA;   // [npp][3]
  const double* K;
  const float* Kf;
  const int4* ao4;    // optional: (AO of A | (A == B) << 30, AO of B, block offset lo, hi)
  const float4* pf8;  // optional: per primitive pair (zeta, PA xyz), (1/(2 zeta), K, 0, 0)
};
