// Drop-in layer for the upstream `_c_ints` extension (include/pychem_gb300.h,
// section 1).  Each entry point takes the host arrays the upstream wrapper received
// (C-contiguous float64, shapes as documented in the header), stages them in one
// device arena, runs one kernel with one thread per output element, copies the
// outputs back and synchronises.  Index conventions follow the upstream kernels
// (Methods/c_ints/*.c): Cartesian components ordered lx descending then ly
// descending (angmom_index.c:3-15), primitive index fastest inside a component
// block, recurrence direction = first non-zero component of the target.
#include <math.h>
#include <string.h>
#include <vector>

#include "../../include/pychem_gb300.h"
#include "common.cuh"
#include "pcg_internal.h"
#include "scat_fund.cuh"

namespace {

__host__ __device__ inline int ncart(int l) { return l < 0 ? 0 : (l + 1) * (l + 2) / 2; }
__host__ __device__ inline int amidx(int x, int y, int z) { int s = y + z; return s * (s + 1) / 2 + z; }
__device__ inline void comp_of(int l, int k, int* c) {
  // inverse of amidx for total l: s = y+z from the triangular index, then z
  int s = 0;
  while ((s + 1) * (s + 2) / 2 <= k) ++s;
  int z = k - s * (s + 1) / 2;
  c[0] = l - s; c[1] = s - z; c[2] = z;
}
__device__ inline int first_nz(const int* c) { return c[0] ? 0 : (c[1] ? 1 : 2); }

// One device allocation for all staged arrays of a call.
struct Arena {
  std::vector<const double*> src;
  std::vector<size_t> n;
  std::vector<double*> dptr;
  double* base = nullptr;
  ~Arena() { if (base) cudaFree(base); }
  int add(const double* h, size_t count) {
    src.push_back(h); n.push_back(count); dptr.push_back(nullptr);
    return (int)src.size() - 1;
  }
  int stage() {
    size_t total = 0;
    for (size_t c : n) total += (c + 31) / 32 * 32;
    if (total == 0) total = 32;
    PCG_CUDA(cudaMalloc(&base, total * sizeof(double)));
    size_t off = 0;
    for (size_t i = 0; i < src.size(); ++i) {
      dptr[i] = base + off;
      if (n[i] && src[i]) PCG_CUDA(cudaMemcpy(dptr[i], src[i], n[i] * sizeof(double), cudaMemcpyHostToDevice));
      off += (n[i] + 31) / 32 * 32;
    }
    return PCG_OK;
  }
  double* d(int i) { return dptr[i]; }
  int fetch(int i, double* h) {
    PCG_CUDA(cudaMemcpy(h, dptr[i], n[i] * sizeof(double), cudaMemcpyDeviceToHost));
    return PCG_OK;
  }
};

inline int grid(long long n) { return (int)((n + 127) / 128 > 65535 * 16 ? 65535 * 16 : (n + 127) / 128); }

#define ARGCHK(cond, msg) do { if (!(cond)) { pcg_set_error(msg); return PCG_ERR_ARG; } } while (0)
#define LAUNCH_DONE() do { PCG_CUDA(cudaGetLastError()); PCG_CUDA(cudaDeviceSynchronize()); } while (0)

// ---------------------------------------------------------------------------------
__global__ void k_shellpair(double* sig, double* ov, double* cen, const double* ae, const double* A, int na,
                            const double* be, const double* B, int nb) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < na * nb; t += gridDim.x * blockDim.x) {
    const int ia = t / nb, ib = t % nb;
    double r2 = 0.0;
    for (int i = 0; i < 3; ++i) r2 += (A[i] - B[i]) * (A[i] - B[i]);
    const double a = ae[ia], b = be[ib], s = 1.0 / (a + b);
    sig[t] = s;
    ov[t] = pow(M_PI * s, 1.5) * exp(-a * b * s * r2);
    for (int i = 0; i < 3; ++i) cen[3 * t + i] = (a * A[i] + b * B[i]) * s;
  }
}

__global__ void k_bound(double* out, const double* CP, const double* CQ, int nla, int nlb, int nlc, int nld) {
  const int n = nla * nlb * nlc * nld;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int ket = t % (nlc * nld), bra = t / (nlc * nld);
    out[t] = sqrt(CP[bra] * CQ[ket]);
  }
}

__global__ void k_fund2(BoysTable bt, double* fund, const double* sP, const double* UP, const double* P,
                        const double* sQ, const double* UQ, const double* Q, double* R, int nbra, int nket,
                        int lmax) {
  const double pf = 0.79788456080286535588;  // sqrt(2/pi)
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nbra * nket; t += gridDim.x * blockDim.x) {
    const int ib = t / nket, ik = t % nket;
    const double U = UP[ib] * UQ[ik];
    const double th2 = 1.0 / (sP[ib] + sQ[ik]);
    double r2 = 0.0;
    for (int i = 0; i < 3; ++i) {
      const double r = P[3 * ib + i] - Q[3 * ik + i];
      R[3 * t + i] = r;
      r2 += r * r;
    }
    double F[PCG_MAXLT + 1];
    if (r2 < 1e-14) {
      for (int m = 0; m <= lmax; ++m) F[m] = 1.0 / (2 * m + 1);
    } else {
      boys_eval_rt(bt, lmax, th2 * r2, F);
    }
    for (int m = 0; m <= lmax; ++m) fund[(size_t)m * nbra * nket + t] = pf * U * pow(2.0 * th2, m + 0.5) * F[m];
  }
}

// j0(S r12) fundamentals in the reference's form (two_electron_scattering.c:6-81):
// U_P U_Q exp(-S^2 (sigma_P + sigma_Q)/4) S^2m z^-m j_m(z), z = S |P - Q|, with its S = 0
// case (U at m = 0, zero above) and R = 0 case (z^-m j_m -> 1/(2m+1)!!).
__global__ void k_fund_scat(double* fund, const double* sP, const double* UP, const double* P, const double* sQ,
                            const double* UQ, const double* Q, double* R, int nbra, int nket, int lmax, double S) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nbra * nket; t += gridDim.x * blockDim.x) {
    const int ib = t / nket, ik = t % nket;
    const double U = UP[ib] * UQ[ik];
    double r2 = 0.0;
    for (int i = 0; i < 3; ++i) {
      const double r = P[3 * ib + i] - Q[3 * ik + i];
      R[3 * t + i] = r;
      r2 += r * r;
    }
    double F[PCG_MAXLT + 1];
    if (S < 1e-14) {
      F[0] = U;
      for (int m = 1; m <= lmax; ++m) F[m] = 0.0;
    } else {
      const double eS = exp(-0.25 * S * S * (sP[ib] + sQ[ik]));
      if (r2 < 1e-14) {
        double df = 1.0;
        for (int m = 0; m <= lmax; ++m) { df *= (double)(2 * m + 1); F[m] = 1.0 / df; }
      } else {
        sph_bessel_scaled_rt(lmax, S * sqrt(r2), F);
      }
      double sp = U * eS;
      for (int m = 0; m <= lmax; ++m) { F[m] *= sp; sp *= S * S; }
    }
    for (int m = 0; m <= lmax; ++m) fund[(size_t)m * nbra * nket + t] = F[m];
  }
}

__global__ void k_vrr2(double* tgt, const double* b0, const double* b1, const double* b2, const double* b3,
                       const double* b4, const double* zeta, const double* eta, const double* kappa,
                       const double* Rx, const double* R, int na, int nb, int nc, int nd, int lbra, int lket,
                       int kidx) {
  const int npb = na * nb, npk = nc * nd;
  const int rows = ncart(lbra) * npb, cols = ncart(lket) * npk, cols4 = ncart(lket - 1) * npk;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < rows * cols; t += gridDim.x * blockDim.x) {
    const int ibra = t / cols, iket = t % cols;
    const int cb = ibra / npb, bp = ibra % npb, ia = bp / nb, ib = bp % nb;
    const int ck = iket / npk, kp = iket % npk, ic = kp / nd, id = kp % nd;
    int e[3], f[3];
    comp_of(lbra, cb, e);
    comp_of(lket, ck, f);
    const int i = first_nz(e);
    int e0[3] = {e[0], e[1], e[2]}; e0[i]--;
    const int ibra0 = amidx(e0[0], e0[1], e0[2]) * npb + bp;
    const double z = zeta[ia * nb + ib];
    const double kap = kidx == 0 ? kappa[ia] : kappa[ib];
    double v = Rx[i] * kap * z * b0[(size_t)ibra0 * cols + iket] + R[3 * ((size_t)bp * npk + kp) + i] * z * b1[(size_t)ibra0 * cols + iket];
    if (e0[i] != 0) {
      int e1[3] = {e0[0], e0[1], e0[2]}; e1[i]--;
      const int ibra1 = amidx(e1[0], e1[1], e1[2]) * npb + bp;
      v += e0[i] * z * (b2[(size_t)ibra1 * cols + iket] - z * b3[(size_t)ibra1 * cols + iket]);
    }
    if (f[i] != 0) {
      int f1[3] = {f[0], f[1], f[2]}; f1[i]--;
      const int iket1 = amidx(f1[0], f1[1], f1[2]) * npk + kp;
      v += f[i] * z * eta[ic * nd + id] * b4[(size_t)ibra0 * cols4 + iket1];
    }
    tgt[t] = v;
  }
}

__global__ void k_contract2(double* out, const double* prim, const double* ccb, const double* cck, int na, int nb,
                            int nc, int nd, int lbra, int lket) {
  const int nbc = ncart(lbra), nkc = ncart(lket), npb = na * nb, npk = nc * nd;
  const int cols = nkc * npk;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nbc * nkc; t += gridDim.x * blockDim.x) {
    const int cb = t / nkc, ck = t % nkc;
    double s = 0.0;
    for (int p = 0; p < npb; ++p)
      for (int q = 0; q < npk; ++q) s += ccb[p] * cck[q] * prim[(size_t)(cb * npb + p) * cols + ck * npk + q];
    out[t] += s;
  }
}

__global__ void k_hrr2(double* tgt, const double* b0, const double* b1, const double* Rx, int la, int lb, int lc,
                       int ld, int goofy) {
  const int nket = ncart(lc) * ncart(ld);
  int lat, lbt, nlb0, nlb1;
  if (goofy == 0) { lat = la; lbt = lb + 1; nlb0 = ncart(lb); nlb1 = ncart(lb); }
  else { lat = la + 1; lbt = lb; nlb0 = ncart(lb + 1) - 1; nlb1 = ncart(lb); }
  const int nbt = ncart(lbt);
  const int rows = ncart(lat) * nbt;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < rows * nket; t += gridDim.x * blockDim.x) {
    const int ibra = t / nket, iket = t % nket;
    int a[3], b[3];
    comp_of(lat, ibra / nbt, a);
    comp_of(lbt, ibra % nbt, b);
    int ia0, ib0, ia1, ib1, i;
    if (goofy == 0) {
      i = first_nz(b);
      int bm[3] = {b[0], b[1], b[2]}; bm[i]--;
      int ap[3] = {a[0], a[1], a[2]}; ap[i]++;
      ia0 = amidx(ap[0], ap[1], ap[2]); ib0 = amidx(bm[0], bm[1], bm[2]);
      ia1 = amidx(a[0], a[1], a[2]); ib1 = ib0;
    } else {
      i = first_nz(a);
      int am[3] = {a[0], a[1], a[2]}; am[i]--;
      int bp[3] = {b[0], b[1], b[2]}; bp[i]++;
      ia0 = amidx(am[0], am[1], am[2]); ib0 = amidx(bp[0], bp[1], bp[2]);
      ia1 = ia0; ib1 = amidx(b[0], b[1], b[2]);
    }
    tgt[t] = b0[(size_t)(ia0 * nlb0 + ib0) * nket + iket] + Rx[i] * b1[(size_t)(ia1 * nlb1 + ib1) * nket + iket];
  }
}

__global__ void k_fund1(BoysTable bt, double* fund, const double* sP, const double* UP, const double* P,
                        const double* Rc, double Z, int n, int lmax) {
  const double pf = -Z * 0.79788456080286535588;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    double r2 = 0.0;
    for (int i = 0; i < 3; ++i) { const double r = P[3 * t + i] - Rc[i]; r2 += r * r; }
    const double zeta = 1.0 / sP[t];
    const double spf = pf * UP[t] * sqrt(2.0 * zeta);
    double F[PCG_MAXLT + 1];
    if (r2 < 1e-14) {
      for (int m = 0; m <= lmax; ++m) F[m] = 1.0 / (2 * m + 1);
    } else {
      boys_eval_rt(bt, lmax, zeta * r2, F);
    }
    for (int m = 0; m <= lmax; ++m) fund[(size_t)m * n + t] = spf * F[m];
  }
}

__global__ void k_vrr1(double* tgt, const double* b0, const double* b1, const double* b2, const double* b3,
                       const double* sP, const double* P, const double* Ra, const double* Rc, int na, int nb,
                       int la, int aux) {
  const int rows = ncart(la) * na;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < rows * nb; t += gridDim.x * blockDim.x) {
    const int ibra = t / nb, ib = t % nb;
    const int ca = ibra / na, ia = ibra % na;
    int a[3];
    comp_of(la, ca, a);
    const int i = first_nz(a);
    int a0[3] = {a[0], a[1], a[2]}; a0[i]--;
    const int ibra0 = amidx(a0[0], a0[1], a0[2]) * na + ia;
    const int pp = ia * nb + ib;
    const double pa = P[3 * pp + i] - Ra[i];
    double v;
    if (aux == 0) {
      v = pa * b0[ibra0 * nb + ib];
      if (a0[i] != 0) {
        int a1[3] = {a0[0], a0[1], a0[2]}; a1[i]--;
        const int ibra1 = amidx(a1[0], a1[1], a1[2]) * na + ia;
        v += a0[i] * 0.5 * sP[pp] * b1[ibra1 * nb + ib];
      }
    } else {
      v = pa * b0[ibra0 * nb + ib] - (P[3 * pp + i] - Rc[i]) * b1[ibra0 * nb + ib];
      if (a0[i] != 0) {
        int a1[3] = {a0[0], a0[1], a0[2]}; a1[i]--;
        const int ibra1 = amidx(a1[0], a1[1], a1[2]) * na + ia;
        v += a0[i] * 0.5 * sP[pp] * (b2[ibra1 * nb + ib] - b3[ibra1 * nb + ib]);
      }
    }
    tgt[t] = v;
  }
}

__global__ void k_hrr1(double* tgt, const double* b0, const double* b1, const double* Rab, int na, int nb, int la,
                       int lb) {
  const int rows = ncart(la) * na, cols = ncart(lb) * nb, cols0 = ncart(lb - 1) * nb;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < rows * cols; t += gridDim.x * blockDim.x) {
    const int r = t / cols, c = t % cols;
    const int ca = r / na, ia = r % na, cb = c / nb, ib = c % nb;
    int a[3], b[3];
    comp_of(la, ca, a);
    comp_of(lb, cb, b);
    const int i = first_nz(b);
    int bm[3] = {b[0], b[1], b[2]}; bm[i]--;
    int ap[3] = {a[0], a[1], a[2]}; ap[i]++;
    const int ib0 = amidx(bm[0], bm[1], bm[2]) * nb + ib;
    const int ia1 = amidx(ap[0], ap[1], ap[2]) * na + ia;
    tgt[t] = b0[(size_t)ia1 * cols0 + ib0] + Rab[i] * b1[(size_t)r * cols0 + ib0];
  }
}

__global__ void k_kinetic(double* tgt, const double* b0, const double* b1, const double* b2, const double* exB,
                          int na, int nb, int la, int lb) {
  const int rows = ncart(la) * na, cols = ncart(lb) * nb;
  const int c0 = ncart(lb + 2) * nb, c2 = ncart(lb - 2) * nb;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < rows * cols; t += gridDim.x * blockDim.x) {
    const int r = t / cols, c = t % cols;
    const int cb = c / nb, ib = c % nb;
    int b[3];
    comp_of(lb, cb, b);
    const double beta = exB[ib];
    double v = beta * (2 * b[0] + 2 * b[1] + 2 * b[2] + 3) * b1[(size_t)r * cols + c];
    double s2 = 0.0;
    for (int i = 0; i < 3; ++i) {
      int bp[3] = {b[0], b[1], b[2]}; bp[i] += 2;
      s2 += b0[(size_t)r * c0 + amidx(bp[0], bp[1], bp[2]) * nb + ib];
    }
    v -= 2 * beta * beta * s2;
    for (int i = 0; i < 3; ++i)
      if (b[i] > 1) {
        int bm[3] = {b[0], b[1], b[2]}; bm[i] -= 2;
        v -= 0.5 * b[i] * (b[i] - 1) * b2[(size_t)r * c2 + amidx(bm[0], bm[1], bm[2]) * nb + ib];
      }
    tgt[t] = v;
  }
}

__global__ void k_contract1(double* out, const double* base, const double* cc, int na, int nb, int la, int lb) {
  const int nca = ncart(la), ncb = ncart(lb), cols = ncb * nb;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nca * ncb; t += gridDim.x * blockDim.x) {
    const int ca = t / ncb, cb = t % ncb;
    double s = 0.0;
    for (int ia = 0; ia < na; ++ia)
      for (int ib = 0; ib < nb; ++ib) s += cc[ia * nb + ib] * base[(size_t)(ca * na + ia) * cols + cb * nb + ib];
    out[t] += s;
  }
}

}  // namespace

extern "C" {

int pcg_shellpair_quantities(double* sigmas, double* overlaps, double* centres, const double* alpha_exps,
                             const double* A, int n_alpha, const double* beta_exps, const double* B, int n_beta) {
  ARGCHK(n_alpha > 0 && n_beta > 0 && sigmas && overlaps && centres, "shellpair_quantities: bad arguments");
  const size_t n = (size_t)n_alpha * n_beta;
  Arena ar;
  int s = ar.add(nullptr, n), o = ar.add(nullptr, n), c = ar.add(nullptr, 3 * n);
  int ea = ar.add(alpha_exps, n_alpha), pa = ar.add(A, 3), eb = ar.add(beta_exps, n_beta), pb = ar.add(B, 3);
  if (int rc = ar.stage()) return rc;
  k_shellpair<<<grid(n), 128>>>(ar.d(s), ar.d(o), ar.d(c), ar.d(ea), ar.d(pa), n_alpha, ar.d(eb), ar.d(pb), n_beta);
  LAUNCH_DONE();
  if (int rc = ar.fetch(s, sigmas)) return rc;
  if (int rc = ar.fetch(o, overlaps)) return rc;
  return ar.fetch(c, centres);
}

int pcg_two_electron_bound(double* bounds, const double* C_P, const double* C_Q, int nla, int nlb, int nlc, int nld) {
  ARGCHK(nla > 0 && nlb > 0 && nlc > 0 && nld > 0 && bounds, "two_electron_bound: bad arguments");
  const size_t n = (size_t)nla * nlb * nlc * nld;
  Arena ar;
  int o = ar.add(nullptr, n), p = ar.add(C_P, (size_t)nla * nlb), q = ar.add(C_Q, (size_t)nlc * nld);
  if (int rc = ar.stage()) return rc;
  k_bound<<<grid(n), 128>>>(ar.d(o), ar.d(p), ar.d(q), nla, nlb, nlc, nld);
  LAUNCH_DONE();
  return ar.fetch(o, bounds);
}

int pcg_two_electron_fundamentals(double* fundamentals, const double* sigma_P, const double* U_P, const double* P,
                                  const double* sigma_Q, const double* U_Q, const double* Q, double* R, int na,
                                  int nb, int nc, int nd, int m, int ints_type, double grid_value) {
  ARGCHK(na > 0 && nb > 0 && nc > 0 && nd > 0 && m >= 0, "two_electron_fundamentals: bad arguments");
  if (m > PCG_MAXLT) { pcg_set_error("two_electron_fundamentals: Boys order above 8 (shells above d)"); return PCG_ERR_UNSUPPORTED; }
  // ints_type 1: j0(S r12) scattering operator at S = grid_value; anything else: 1/r12
  // (the reference's branch, _c_ints.c:236-240)
  if (ints_type == 1 && !(grid_value >= 0.0)) {
    pcg_set_error("two_electron_fundamentals: scattering needs grid_value >= 0");
    return PCG_ERR_ARG;
  }
  BoysTable bt;
  if (ints_type != 1)
    if (int rc = pcg_ensure_boys(&bt)) return rc;
  const size_t nbra = (size_t)na * nb, nket = (size_t)nc * nd;
  Arena ar;
  int f = ar.add(nullptr, (m + 1) * nbra * nket), r = ar.add(nullptr, 3 * nbra * nket);
  int sp = ar.add(sigma_P, nbra), up = ar.add(U_P, nbra), pp = ar.add(P, 3 * nbra);
  int sq = ar.add(sigma_Q, nket), uq = ar.add(U_Q, nket), qq = ar.add(Q, 3 * nket);
  if (int rc = ar.stage()) return rc;
  if (ints_type == 1)
    k_fund_scat<<<grid(nbra * nket), 128>>>(ar.d(f), ar.d(sp), ar.d(up), ar.d(pp), ar.d(sq), ar.d(uq), ar.d(qq),
                                            ar.d(r), (int)nbra, (int)nket, m, grid_value);
  else
    k_fund2<<<grid(nbra * nket), 128>>>(bt, ar.d(f), ar.d(sp), ar.d(up), ar.d(pp), ar.d(sq), ar.d(uq), ar.d(qq),
                                        ar.d(r), (int)nbra, (int)nket, m);
  LAUNCH_DONE();
  if (int rc = ar.fetch(f, fundamentals)) return rc;
  return ar.fetch(r, R);
}

int pcg_two_electron_vrr(double* target, const double* base0, const double* base1, const double* base2,
                         const double* base3, const double* base4, const double* zeta, const double* eta,
                         const double* kappa, const double* Rx, const double* R, int na, int nb, int nc, int nd,
                         int lbra, int lket, int kappa_index) {
  ARGCHK(na > 0 && nb > 0 && nc > 0 && nd > 0 && lbra >= 1 && lket >= 0 && target && base0 && base1,
         "two_electron_vrr: bad arguments");
  ARGCHK(lbra < 2 || (base2 && base3), "two_electron_vrr: base2/base3 required for lbra >= 2");
  ARGCHK(lket < 1 || base4, "two_electron_vrr: base4 required for lket >= 1");
  const size_t npb = (size_t)na * nb, npk = (size_t)nc * nd;
  const size_t cols = ncart(lket) * npk;
  Arena ar;
  int t = ar.add(nullptr, ncart(lbra) * npb * cols);
  int b0 = ar.add(base0, ncart(lbra - 1) * npb * cols), b1 = ar.add(base1, ncart(lbra - 1) * npb * cols);
  int b2 = ar.add(lbra >= 2 ? base2 : nullptr, lbra >= 2 ? ncart(lbra - 2) * npb * cols : 0);
  int b3 = ar.add(lbra >= 2 ? base3 : nullptr, lbra >= 2 ? ncart(lbra - 2) * npb * cols : 0);
  int b4 = ar.add(lket >= 1 ? base4 : nullptr, lket >= 1 ? ncart(lbra - 1) * npb * ncart(lket - 1) * npk : 0);
  int z = ar.add(zeta, npb), e = ar.add(eta, npk), k = ar.add(kappa, kappa_index == 0 ? na : nb);
  int rx = ar.add(Rx, 3), r = ar.add(R, 3 * npb * npk);
  if (int rc = ar.stage()) return rc;
  const long long n = (long long)ncart(lbra) * npb * cols;
  k_vrr2<<<grid(n), 128>>>(ar.d(t), ar.d(b0), ar.d(b1), ar.d(b2), ar.d(b3), ar.d(b4), ar.d(z), ar.d(e), ar.d(k),
                           ar.d(rx), ar.d(r), na, nb, nc, nd, lbra, lket, kappa_index);
  LAUNCH_DONE();
  return ar.fetch(t, target);
}

int pcg_two_electron_contract(double* contracted, const double* primitive, const double* cc_bra,
                              const double* cc_ket, int na, int nb, int nc, int nd, int lbra, int lket) {
  ARGCHK(na > 0 && nb > 0 && nc > 0 && nd > 0 && lbra >= 0 && lket >= 0 && contracted && primitive,
         "two_electron_contract: bad arguments");
  const size_t npb = (size_t)na * nb, npk = (size_t)nc * nd;
  Arena ar;
  int o = ar.add(contracted, (size_t)ncart(lbra) * ncart(lket));
  int p = ar.add(primitive, ncart(lbra) * npb * ncart(lket) * npk);
  int cb = ar.add(cc_bra, npb), ck = ar.add(cc_ket, npk);
  if (int rc = ar.stage()) return rc;
  k_contract2<<<grid((long long)ncart(lbra) * ncart(lket)), 128>>>(ar.d(o), ar.d(p), ar.d(cb), ar.d(ck), na, nb,
                                                                   nc, nd, lbra, lket);
  LAUNCH_DONE();
  return ar.fetch(o, contracted);
}

int pcg_two_electron_hrr(double* target, const double* base0, const double* base1, const double* Rx, int la, int lb,
                         int lc, int ld, int goofy) {
  ARGCHK(la >= 0 && lb >= 0 && lc >= 0 && ld >= 0 && (goofy == 0 || goofy == 1) && target && base0 && base1,
         "two_electron_hrr: bad arguments");
  const size_t nket = (size_t)ncart(lc) * ncart(ld);
  const size_t rows_t = goofy == 0 ? (size_t)ncart(la) * ncart(lb + 1) : (size_t)ncart(la + 1) * ncart(lb);
  const size_t rows0 = goofy == 0 ? (size_t)ncart(la + 1) * ncart(lb) : (size_t)ncart(la) * ncart(lb + 1);
  const size_t rows1 = (size_t)ncart(la) * ncart(lb);
  Arena ar;
  int t = ar.add(nullptr, rows_t * nket), b0 = ar.add(base0, rows0 * nket), b1 = ar.add(base1, rows1 * nket);
  int rx = ar.add(Rx, 3);
  if (int rc = ar.stage()) return rc;
  k_hrr2<<<grid(rows_t * nket), 128>>>(ar.d(t), ar.d(b0), ar.d(b1), ar.d(rx), la, lb, lc, ld, goofy);
  LAUNCH_DONE();
  return ar.fetch(t, target);
}

int pcg_one_electron_fundamentals(double* fundamentals, const double* sigma_P, const double* U_P, const double* P,
                                  const double* Rc, double Z, int na, int nb, int m) {
  ARGCHK(na > 0 && nb > 0 && m >= 0 && fundamentals, "one_electron_fundamentals: bad arguments");
  if (m > PCG_MAXLT) { pcg_set_error("one_electron_fundamentals: Boys order above 8"); return PCG_ERR_UNSUPPORTED; }
  BoysTable bt;
  if (int rc = pcg_ensure_boys(&bt)) return rc;
  const size_t n = (size_t)na * nb;
  Arena ar;
  int f = ar.add(nullptr, (m + 1) * n), s = ar.add(sigma_P, n), u = ar.add(U_P, n), p = ar.add(P, 3 * n);
  int c = ar.add(Rc, 3);
  if (int rc = ar.stage()) return rc;
  k_fund1<<<grid(n), 128>>>(bt, ar.d(f), ar.d(s), ar.d(u), ar.d(p), ar.d(c), Z, (int)n, m);
  LAUNCH_DONE();
  return ar.fetch(f, fundamentals);
}

int pcg_one_electron_vrr(double* target, const double* const* base_list, const double* sigma_P, const double* P,
                         const double* Ra, const double* Rc, int atom_index, int n_base, int na, int nb, int la) {
  ARGCHK(na > 0 && nb > 0 && la >= 1 && n_base >= 1 && base_list && target, "one_electron_vrr: bad arguments");
  const int aux = atom_index == -1 ? 0 : 1;
  const size_t n1 = (size_t)ncart(la - 1) * na * nb, n2 = (size_t)ncart(la - 2) * na * nb;
  const double* b0 = base_list[0];
  const double* b1 = n_base > 1 ? base_list[1] : nullptr;
  const double* b2 = n_base == 4 ? base_list[2] : nullptr;
  const double* b3 = n_base == 4 ? base_list[3] : nullptr;
  if (aux == 0) ARGCHK(la < 2 || b1, "one_electron_vrr: overlap needs two base classes for la >= 2");
  else ARGCHK(b1 && (la < 2 || (b2 && b3)), "one_electron_vrr: nuclear attraction needs 2 (la=1) or 4 base classes");
  Arena ar;
  int t = ar.add(nullptr, (size_t)ncart(la) * na * nb);
  int i0 = ar.add(b0, n1);
  int i1 = ar.add(b1, b1 ? (aux == 0 ? n2 : n1) : 0);
  int i2 = ar.add(b2, b2 ? n2 : 0), i3 = ar.add(b3, b3 ? n2 : 0);
  int s = ar.add(sigma_P, (size_t)na * nb), p = ar.add(P, 3 * (size_t)na * nb), ra = ar.add(Ra, 3);
  int rc_ = ar.add(aux ? Rc : nullptr, aux ? 3 : 0);
  if (int rc = ar.stage()) return rc;
  k_vrr1<<<grid((long long)ncart(la) * na * nb), 128>>>(ar.d(t), ar.d(i0), ar.d(i1), ar.d(i2), ar.d(i3), ar.d(s),
                                                        ar.d(p), ar.d(ra), ar.d(rc_), na, nb, la, aux);
  LAUNCH_DONE();
  return ar.fetch(t, target);
}

int pcg_one_electron_hrr(double* target, const double* const* base_list, const double* Rab, int n_base, int na,
                         int nb, int la, int lb) {
  ARGCHK(na > 0 && nb > 0 && la >= 0 && lb >= 1 && n_base == 2 && base_list && target,
         "one_electron_hrr: bad arguments");
  const size_t cols0 = (size_t)ncart(lb - 1) * nb;
  Arena ar;
  int t = ar.add(nullptr, (size_t)ncart(la) * na * ncart(lb) * nb);
  int b0 = ar.add(base_list[0], (size_t)ncart(la + 1) * na * cols0), b1 = ar.add(base_list[1], (size_t)ncart(la) * na * cols0);
  int r = ar.add(Rab, 3);
  if (int rc = ar.stage()) return rc;
  k_hrr1<<<grid((long long)ncart(la) * na * ncart(lb) * nb), 128>>>(ar.d(t), ar.d(b0), ar.d(b1), ar.d(r), na, nb,
                                                                    la, lb);
  LAUNCH_DONE();
  return ar.fetch(t, target);
}

int pcg_one_electron_kinetic(double* target, const double* const* base_list, const double* exB, int n_base, int na,
                             int nb, int la, int lb) {
  ARGCHK(na > 0 && nb > 0 && la >= 0 && lb >= 0 && n_base >= 2 && base_list && target,
         "one_electron_kinetic: bad arguments");
  ARGCHK(lb < 2 || n_base >= 3, "one_electron_kinetic: lb >= 2 needs the [a|b-2] class");
  const size_t rows = (size_t)ncart(la) * na;
  Arena ar;
  int t = ar.add(nullptr, rows * ncart(lb) * nb);
  int b0 = ar.add(base_list[0], rows * ncart(lb + 2) * nb), b1 = ar.add(base_list[1], rows * ncart(lb) * nb);
  int b2 = ar.add(lb >= 2 ? base_list[2] : nullptr, lb >= 2 ? rows * ncart(lb - 2) * nb : 0);
  int e = ar.add(exB, nb);
  if (int rc = ar.stage()) return rc;
  k_kinetic<<<grid((long long)rows * ncart(lb) * nb), 128>>>(ar.d(t), ar.d(b0), ar.d(b1), ar.d(b2), ar.d(e), na, nb,
                                                             la, lb);
  LAUNCH_DONE();
  return ar.fetch(t, target);
}

int pcg_one_electron_contract(double* target, const double* base, const double* cc, int na, int nb, int la, int lb) {
  ARGCHK(na > 0 && nb > 0 && la >= 0 && lb >= 0 && target && base, "one_electron_contract: bad arguments");
  Arena ar;
  int o = ar.add(target, (size_t)ncart(la) * ncart(lb));
  int b = ar.add(base, (size_t)ncart(la) * na * ncart(lb) * nb), c = ar.add(cc, (size_t)na * nb);
  if (int rc = ar.stage()) return rc;
  k_contract1<<<grid((long long)ncart(la) * ncart(lb)), 128>>>(ar.d(o), ar.d(b), ar.d(c), na, nb, la, lb);
  LAUNCH_DONE();
  return ar.fetch(o, target);
}

}  // extern "C"
