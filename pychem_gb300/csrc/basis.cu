// Boys table, primitive-pair data and one-electron (S, T, V) kernels.
//
// Upstream counterparts: pair data Methods/c_ints/shellpair_quantities.c:5-38 and
// Util/structures.py:918-956; one-electron integrals Methods/integrals.py:220-370 with
// one_electron_{fundamentals,vrr,hrr,kinetic,contract}.c; core/overlap assembly
// Methods/hartree_fock.py:207-224.
#include <math.h>
#include <stdio.h>
#include <string.h>
#include <vector>

#include "common.cuh"
#include "pcg_internal.h"

// ----------------------------------------------------------------------------------
// Boys table (host build once per device)
// ----------------------------------------------------------------------------------
static void boys_host(int mmax, double T, double* F) {
  // positive series for the top order, downward recursion (stable for all T here,
  // T <= 48 keeps exp(T) finite)
  double e = exp(-T);
  double term = 1.0 / (2 * mmax + 1), acc = term;
  for (int k = 1; k < 10000; ++k) {
    term *= 2.0 * T / (2 * mmax + 2 * k + 1);
    acc += term;
    if (k > 10 && term < 1e-18 * acc) break;
  }
  F[mmax] = e * acc;
  for (int m = mmax; m > 0; --m) F[m - 1] = (2.0 * T * F[m] + e) / (2 * m - 1);
}

static DeviceState g_dev[16];

DeviceState* pcg_state() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 16) return nullptr;
  return &g_dev[dev];
}

int pcg_ensure_boys(BoysTable* out) {
  DeviceState* st = pcg_state();
  if (!st) { pcg_set_error("no CUDA device"); return PCG_ERR_CUDA; }
  if (!st->boys_c) {
    const int nm = BOYS_M + BOYS_K;
    std::vector<double> c((size_t)BOYS_NP * BOYS_M * BOYS_K), ex(BOYS_NP);
    std::vector<float> cf((size_t)BOYS_NP * BOYS_M * BOYS_KF), exf(BOYS_NP);
    double F[64], fact[BOYS_K];
    fact[0] = 1.0;
    for (int k = 1; k < BOYS_K; ++k) fact[k] = fact[k - 1] * k;
    for (int p = 0; p < BOYS_NP; ++p) {
      double T = (double)p / BOYS_INV_H;
      boys_host(nm, T, F);
      for (int m = 0; m < BOYS_M; ++m) {
        for (int k = 0; k < BOYS_K; ++k) c[((size_t)p * BOYS_M + m) * BOYS_K + k] = F[m + k] / fact[k];
        for (int k = 0; k < BOYS_KF; ++k) cf[((size_t)p * BOYS_M + m) * BOYS_KF + k] = (float)(F[m + k] / fact[k]);
      }
      ex[p] = exp(-T);
      exf[p] = (float)ex[p];
    }
    double *dc = nullptr, *dex = nullptr;
    float *dcf = nullptr, *dexf = nullptr;
    PCG_CUDA(cudaMalloc(&dc, c.size() * sizeof(double)));
    PCG_CUDA(cudaMalloc(&dex, ex.size() * sizeof(double)));
    PCG_CUDA(cudaMalloc(&dcf, cf.size() * sizeof(float)));
    PCG_CUDA(cudaMalloc(&dexf, exf.size() * sizeof(float)));
    PCG_CUDA(cudaMemcpy(dc, c.data(), c.size() * sizeof(double), cudaMemcpyHostToDevice));
    PCG_CUDA(cudaMemcpy(dex, ex.data(), ex.size() * sizeof(double), cudaMemcpyHostToDevice));
    PCG_CUDA(cudaMemcpy(dcf, cf.data(), cf.size() * sizeof(float), cudaMemcpyHostToDevice));
    PCG_CUDA(cudaMemcpy(dexf, exf.data(), exf.size() * sizeof(float), cudaMemcpyHostToDevice));
    st->boys_c = dc; st->boys_ex = dex; st->boys_cf = dcf; st->boys_exf = dexf;
  }
  out->c = st->boys_c; out->ex = st->boys_ex; out->cf = st->boys_cf; out->exf = st->boys_exf;
  return PCG_OK;
}

// ----------------------------------------------------------------------------------
// Primitive-pair data: one thread per shell pair, loop over its primitive pairs.
// ----------------------------------------------------------------------------------
__global__ void k_pair_data(DevBasis b, int npair, const int* pA, const int* pB, const int* ppoff,
                            double* AB, double* zeta, double* P, double* PA, double* K, float* Kf,
                            double* oo2z) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npair) return;
  const int A = pA[p], B = pB[p];
  const double ax = b.sh_xyz[3 * A], ay = b.sh_xyz[3 * A + 1], az = b.sh_xyz[3 * A + 2];
  const double bx = b.sh_xyz[3 * B], by = b.sh_xyz[3 * B + 1], bz = b.sh_xyz[3 * B + 2];
  const double dx = ax - bx, dy = ay - by, dz = az - bz;
  const double r2 = dx * dx + dy * dy + dz * dz;
  AB[3 * p] = dx; AB[3 * p + 1] = dy; AB[3 * p + 2] = dz;
  const int na = b.sh_nprim[A], nb = b.sh_nprim[B];
  int k = ppoff[p];
  for (int i = 0; i < na; ++i) {
    const double a = b.pr_exp[b.sh_prim[A] + i], ca = b.pr_cc[b.sh_prim[A] + i];
    for (int j = 0; j < nb; ++j, ++k) {
      const double be = b.pr_exp[b.sh_prim[B] + j], cb = b.pr_cc[b.sh_prim[B] + j];
      const double z = a + be, s = 1.0 / z;
      const double U = pow(M_PI * s, 1.5) * exp(-a * be * s * r2);
      const double px = (a * ax + be * bx) * s, py = (a * ay + be * by) * s, pz = (a * az + be * bz) * s;
      zeta[k] = z;
      oo2z[k] = 0.5 * s;
      P[3 * k] = px; P[3 * k + 1] = py; P[3 * k + 2] = pz;
      PA[3 * k] = px - ax; PA[3 * k + 1] = py - ay; PA[3 * k + 2] = pz - az;
      // sqrt(2/sqrt(pi)) = 1.0622519320271968
      const double kk = ca * cb * 1.0622519320271968 * U * sqrt(z);
      K[k] = kk;
      Kf[k] = (float)kk;
    }
  }
}

int pcg_launch_pair_data(const DevBasis& b, int npair, const int* pA, const int* pB, const int* ppoff,
                         double* AB, double* zeta, double* P, double* PA, double* K, float* Kf, double* oo2z,
                         cudaStream_t s) {
  if (npair <= 0) return PCG_OK;
  k_pair_data<<<(npair + 127) / 128, 128, 0, s>>>(b, npair, pA, pB, ppoff, AB, zeta, P, PA, K, Kf, oo2z);
  PCG_CUDA(cudaGetLastError());
  return PCG_OK;
}

__global__ void k_pair_data_f32(int npp, const double* __restrict__ zeta, const double* __restrict__ PA,
                                const double* __restrict__ oo2z, const float* __restrict__ Kf,
                                float4* __restrict__ pf8) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= npp) return;
  pf8[2 * k] = make_float4((float)zeta[k], (float)PA[3 * k], (float)PA[3 * k + 1], (float)PA[3 * k + 2]);
  pf8[2 * k + 1] = make_float4((float)oo2z[k], Kf[k], 0.0f, 0.0f);
}

int pcg_launch_pair_data_f32(int npp, const double* zeta, const double* PA, const double* oo2z, const float* Kf,
                             float* pf8, cudaStream_t s) {
  if (npp <= 0) return PCG_OK;
  k_pair_data_f32<<<(npp + 255) / 256, 256, 0, s>>>(npp, zeta, PA, oo2z, Kf, (float4*)pf8);
  PCG_CUDA(cudaGetLastError());
  return PCG_OK;
}

__global__ void k_pair_ao(DevBasis b, int npair, const int* __restrict__ pA, const int* __restrict__ pB,
                          int4* __restrict__ ao4) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npair) return;
  const int A = pA[p], B = pB[p];
  const long long o = dev_blk(b, A);
  ao4[p] = make_int4(b.sh_ao[A] | (A == B ? 1 << 30 : 0), b.sh_ao[B], (int)(unsigned)(o & 0xFFFFFFFFll),
                     (int)(o >> 32));
}

int pcg_launch_pair_ao(const DevBasis& b, int npair, const int* pA, const int* pB, int* ao4, cudaStream_t s) {
  if (npair <= 0) return PCG_OK;
  k_pair_ao<<<(npair + 127) / 128, 128, 0, s>>>(b, npair, pA, pB, (int4*)ao4);
  PCG_CUDA(cudaGetLastError());
  return PCG_OK;
}

// ----------------------------------------------------------------------------------
// One-electron integrals
// ----------------------------------------------------------------------------------
__device__ __forceinline__ int d_ncart(int l) { return (l + 1) * (l + 2) / 2; }
__device__ __forceinline__ int d_off(int l) { return l * (l + 1) * (l + 2) / 6; }
__device__ __forceinline__ int d_gidx(int x, int y, int z) {
  int l = x + y + z, s = y + z;
  return d_off(l) + s * (s + 1) / 2 + z;
}
__device__ __forceinline__ void d_comp(int l, int k, int* c) {
  // k-th Cartesian component of shell l (lx descending, then ly descending)
  int idx = 0;
  for (int lx = l; lx >= 0; --lx)
    for (int ly = l - lx; ly >= 0; --ly) {
      if (idx == k) { c[0] = lx; c[1] = ly; c[2] = l - lx - ly; return; }
      ++idx;
    }
}

// Cartesian -> spherical row coefficient times the component normalisation ratio.
__device__ __forceinline__ double d_sph(int l, int r, int c) {
  if (l <= 1) return r == c ? 1.0 : 0.0;
  // d: xx xy xz yy yz zz; ratio sqrt(3) for the mixed components xy, xz, yz
  const double h = 0.86602540378443864676, s3 = 1.7320508075688772935;
  switch (r) {
    case 0: return c == 0 ? h : (c == 3 ? -h : 0.0);
    case 1: return c == 1 ? s3 : 0.0;
    case 2: return c == 2 ? s3 : 0.0;
    case 3: return c == 4 ? s3 : 0.0;
    default: return c == 0 ? -0.5 : (c == 3 ? -0.5 : (c == 5 ? 1.0 : 0.0));
  }
}

// One warp per shell pair: lanes stride over the primitive pairs for S and T and over
// (primitive pair, nucleus) items for the nuclear attraction V (the loop that
// dominates: nuclei x primitive pairs), the Cartesian blocks are summed across the
// warp with shuffles, and lane 0 applies the spherical transform and stores both
// triangles of S and H (Methods/integrals.py:220-370).
struct OePrim {
  double U, z, oo2z, cc, P[3], PA[3], PB[3];
};

__device__ __forceinline__ OePrim oe_prim(const DevBasis& b, int A, int B, int ia, int ib, double r2) {
  OePrim q;
  const double* Ax = b.sh_xyz + 3 * A;
  const double* Bx = b.sh_xyz + 3 * B;
  const double al = b.pr_exp[b.sh_prim[A] + ia], be = b.pr_exp[b.sh_prim[B] + ib];
  q.cc = b.pr_cc[b.sh_prim[A] + ia] * b.pr_cc[b.sh_prim[B] + ib];
  q.z = al + be;
  const double s = 1.0 / q.z;
  q.oo2z = 0.5 * s;
  q.U = pow(M_PI * s, 1.5) * exp(-al * be * s * r2);
  for (int i = 0; i < 3; ++i) {
    q.P[i] = (al * Ax[i] + be * Bx[i]) * s;
    q.PA[i] = q.P[i] - Ax[i];
    q.PB[i] = q.P[i] - Bx[i];
  }
  return q;
}

__global__ void k_one_electron(DevBasis b, BoysTable bt, int npair, const int* pA, const int* pB,
                               double* S, double* H) {
  const int p = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (p >= npair) return;  // whole warps leave together
  const int A = pA[p], B = pB[p];
  const int la = b.sh_l[A], lb = b.sh_l[B];
  const int nca = d_ncart(la), ncb = d_ncart(lb);
  double Sc[36], Tc[36], Vc[36];
  for (int i = 0; i < 36; ++i) { Sc[i] = 0.0; Tc[i] = 0.0; Vc[i] = 0.0; }
  const double* Ax = b.sh_xyz + 3 * A;
  const double* Bx = b.sh_xyz + 3 * B;
  double r2 = 0.0;
  for (int i = 0; i < 3; ++i) r2 += (Ax[i] - Bx[i]) * (Ax[i] - Bx[i]);
  const int npa = b.sh_nprim[A], npb = b.sh_nprim[B];
  for (int item = lane; item < npa * npb; item += 32) {
    const int ia = item / npb, ib = item % npb;
    const double be = b.pr_exp[b.sh_prim[B] + ib];
    const OePrim q = oe_prim(b, A, B, ia, ib, r2);
    const double U = q.U, oo2z = q.oo2z, cc = q.cc;
    const double *PA = q.PA, *PB = q.PB;
      // 1D overlap factors E[dir][i][j], i <= la, j <= lb + 2 (Obara-Saika)
      double E[3][3][5];
      for (int d = 0; d < 3; ++d) {
        for (int i = 0; i <= la; ++i)
          for (int j = 0; j <= lb + 2; ++j) {
            double v;
            if (i == 0 && j == 0) v = 1.0;
            else if (j == 0) {
              v = PA[d] * E[d][i - 1][0];
              if (i > 1) v += (i - 1) * oo2z * E[d][i - 2][0];
            } else {
              v = PB[d] * E[d][i][j - 1];
              if (i > 0) v += i * oo2z * E[d][i - 1][j - 1];
              if (j > 1) v += (j - 1) * oo2z * E[d][i][j - 2];
            }
            E[d][i][j] = v;
          }
      }
      for (int ka = 0; ka < nca; ++ka) {
        int x[3]; d_comp(la, ka, x);
        for (int kb = 0; kb < ncb; ++kb) {
          int y[3]; d_comp(lb, kb, y);
          const double sv = E[0][x[0]][y[0]] * E[1][x[1]][y[1]] * E[2][x[2]][y[2]];
          // kinetic energy from overlaps [a|b+2], [a|b], [a|b-2] (one_electron_kinetic.c:60-64)
          double t = be * (2 * lb + 3) * sv;
          for (int i = 0; i < 3; ++i) {
            int yp[3] = {y[0], y[1], y[2]};
            yp[i] += 2;
            t -= 2.0 * be * be * E[0][x[0]][yp[0]] * E[1][x[1]][yp[1]] * E[2][x[2]][yp[2]];
            if (y[i] > 1) {
              int ym[3] = {y[0], y[1], y[2]};
              ym[i] -= 2;
              t -= 0.5 * y[i] * (y[i] - 1) * E[0][x[0]][ym[0]] * E[1][x[1]][ym[1]] * E[2][x[2]][ym[2]];
            }
          }
          Sc[ka * ncb + kb] += cc * U * sv;
          Tc[ka * ncb + kb] += cc * U * t;
        }
      }
  }
  // nuclear attraction: Obara-Saika with auxiliary index over the molecule's nuclei
  const int L = la + lb;
  const int c0 = b.sh_at0 ? b.sh_at0[A] : 0;
  const int c1 = b.sh_at0 ? c0 + b.sh_nat[A] : b.natom;
  const int nnuc = c1 - c0;
  for (int item = lane; item < npa * npb * nnuc; item += 32) {
    const int c = c0 + item % nnuc, pp = item / nnuc;
    const OePrim q = oe_prim(b, A, B, pp / npb, pp % npb, r2);
    const double U = q.U, oo2z = q.oo2z, cc = q.cc, z = q.z;
    const double *P = q.P, *PA = q.PA, *PB = q.PB;
    {
        const double* C = b.at_xyz + 3 * c;
        double PC[3], pc2 = 0.0;
        for (int i = 0; i < 3; ++i) { PC[i] = P[i] - C[i]; pc2 += PC[i] * PC[i]; }
        double F[PCG_MAXLT + 1];
        boys_eval_rt(bt, L, z * pc2, F);
        const double pre = -b.at_z[c] * 2.0 * sqrt(z * (1.0 / M_PI)) * U * cc;
        double V[10][10][5];  // [a global][b global][m]
        for (int m = 0; m <= L; ++m) V[0][0][m] = pre * F[m];
        for (int l = 1; l <= la; ++l)
          for (int k = 0; k < d_ncart(l); ++k) {
            int a[3]; d_comp(l, k, a);
            int i = a[0] ? 0 : (a[1] ? 1 : 2);
            int am[3] = {a[0], a[1], a[2]}; am[i]--;
            int g = d_gidx(a[0], a[1], a[2]), g1 = d_gidx(am[0], am[1], am[2]);
            int g2 = -1;
            if (am[i] > 0) { int amm[3] = {am[0], am[1], am[2]}; amm[i]--; g2 = d_gidx(amm[0], amm[1], amm[2]); }
            for (int m = 0; m <= L - l; ++m) {
              double v = PA[i] * V[g1][0][m] - PC[i] * V[g1][0][m + 1];
              if (g2 >= 0) v += am[i] * oo2z * (V[g2][0][m] - V[g2][0][m + 1]);
              V[g][0][m] = v;
            }
          }
        for (int lbb = 1; lbb <= lb; ++lbb)
          for (int kb = 0; kb < d_ncart(lbb); ++kb) {
            int bb[3]; d_comp(lbb, kb, bb);
            int i = bb[0] ? 0 : (bb[1] ? 1 : 2);
            int bm[3] = {bb[0], bb[1], bb[2]}; bm[i]--;
            int gb = d_gidx(bb[0], bb[1], bb[2]), gb1 = d_gidx(bm[0], bm[1], bm[2]);
            int gb2 = -1;
            if (bm[i] > 0) { int bmm[3] = {bm[0], bm[1], bm[2]}; bmm[i]--; gb2 = d_gidx(bmm[0], bmm[1], bmm[2]); }
            for (int laa = 0; laa <= la; ++laa)
              for (int ka = 0; ka < d_ncart(laa); ++ka) {
                int a[3]; d_comp(laa, ka, a);
                int ga = d_gidx(a[0], a[1], a[2]);
                int ga1 = -1;
                if (a[i] > 0) { int am[3] = {a[0], a[1], a[2]}; am[i]--; ga1 = d_gidx(am[0], am[1], am[2]); }
                for (int m = 0; m <= L - laa - lbb; ++m) {
                  double v = PB[i] * V[ga][gb1][m] - PC[i] * V[ga][gb1][m + 1];
                  if (ga1 >= 0) v += a[i] * oo2z * (V[ga1][gb1][m] - V[ga1][gb1][m + 1]);
                  if (gb2 >= 0) v += bm[i] * oo2z * (V[ga][gb2][m] - V[ga][gb2][m + 1]);
                  V[ga][gb][m] = v;
                }
              }
          }
        for (int ka = 0; ka < nca; ++ka)
          for (int kb = 0; kb < ncb; ++kb) {
            int x[3], y[3];
            d_comp(la, ka, x);
            d_comp(lb, kb, y);
            Vc[ka * ncb + kb] += V[d_gidx(x[0], x[1], x[2])][d_gidx(y[0], y[1], y[2])][0];
          }
      }
    }
  // sum the lanes' Cartesian blocks
  for (int i = 0; i < nca * ncb; ++i) {
    double sv = Sc[i], tv = Tc[i], vv = Vc[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      sv += __shfl_xor_sync(0xffffffffu, sv, o);
      tv += __shfl_xor_sync(0xffffffffu, tv, o);
      vv += __shfl_xor_sync(0xffffffffu, vv, o);
    }
    Sc[i] = sv; Tc[i] = tv; Vc[i] = vv;
  }
  if (lane != 0) return;
  // spherical transform and store both triangles
  const int nsa = 2 * la + 1, nsb = 2 * lb + 1;
  const int oa = b.sh_ao[A], ob = b.sh_ao[B];
  const int n = b.ld;
  const long long o = b.sh_blk ? b.sh_blk[A] : 0ll;
  S += o;
  H += o;
  for (int r = 0; r < nsa; ++r)
    for (int q = 0; q < nsb; ++q) {
      double s = 0.0, h = 0.0;
      for (int ka = 0; ka < nca; ++ka) {
        const double ca = d_sph(la, r, ka);
        if (ca == 0.0) continue;
        for (int kb = 0; kb < ncb; ++kb) {
          const double cb = d_sph(lb, q, kb);
          if (cb == 0.0) continue;
          s += ca * cb * Sc[ka * ncb + kb];
          h += ca * cb * (Tc[ka * ncb + kb] + Vc[ka * ncb + kb]);
        }
      }
      S[(size_t)(oa + r) * n + ob + q] = s;
      S[(size_t)(ob + q) * n + oa + r] = s;
      H[(size_t)(oa + r) * n + ob + q] = h;
      H[(size_t)(ob + q) * n + oa + r] = h;
    }
}

int pcg_launch_one_electron(const DevBasis& b, const BoysTable& bt, int npair, const int* pA, const int* pB,
                            double* S, double* H, cudaStream_t s) {
  if (npair <= 0) return PCG_OK;
  k_one_electron<<<(unsigned)(((long long)npair * 32 + 127) / 128), 128, 0, s>>>(b, bt, npair, pA, pB, S, H);
  PCG_CUDA(cudaGetLastError());
  return PCG_OK;
}
