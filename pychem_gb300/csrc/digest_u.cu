// Unrestricted Fock digestion (one translation unit of its own: the 21 class
// instantiations compile in parallel with eri.cu).
#include "common.cuh"
#include "pcg_internal.h"

// Unrestricted digestion (Methods/hartree_fock.py:329-355 with D_a != D_b): the J part
// from the half total density Dh = (D_a + D_b)/2 goes to GJ, the exchange parts of
// each spin to GKa and GKb, with the same factors as k_digest, so that
// F_s = H + sym(GJ + GKs) = H + J[D_a + D_b] - K[D_s].
template <int NA, int NB, int NC, int ND>
__global__ void __launch_bounds__(128) k_digest_u(DevBasis b, DevPairsExt pr, const int2* __restrict__ tasks,
                                                  int ntask, const double* __restrict__ store,
                                                  const double* __restrict__ Da, const double* __restrict__ Db,
                                                  double* __restrict__ GJ, double* __restrict__ GKa,
                                                  double* __restrict__ GKb) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntask) return;
  const int2 tk = tasks[t];
  const int A = __ldg(pr.p.A + tk.x), B = __ldg(pr.p.B + tk.x);
  const int C = __ldg(pr.p.A + tk.y), Dd = __ldg(pr.p.B + tk.y);
  const long long o = dev_blk(b, A);
  const int oa = __ldg(b.sh_ao + A), ob = __ldg(b.sh_ao + B), oc = __ldg(b.sh_ao + C), od = __ldg(b.sh_ao + Dd);
  const int n = b.ld;
  Da += o; Db += o; GJ += o; GKa += o; GKb += o;
  const double deg = (A == B ? 1.0 : 2.0) * (C == Dd ? 1.0 : 2.0) * (tk.x == tk.y ? 1.0 : 2.0);
  auto at = [&](const double* M, int i, int j) { return __ldg(M + (size_t)i * n + j); };
  double Hab[NA][NB], Hcd[NC][ND];
  double Aac[NA][NC], Abd[NB][ND], Aad[NA][ND], Abc[NB][NC];
  double Bac[NA][NC], Bbd[NB][ND], Bad[NA][ND], Bbc[NB][NC];
  double gab[NA][NB] = {}, gcd[NC][ND] = {};
  double xac[NA][NC] = {}, xbd[NB][ND] = {}, xad[NA][ND] = {}, xbc[NB][NC] = {};
  double yac[NA][NC] = {}, ybd[NB][ND] = {}, yad[NA][ND] = {}, ybc[NB][NC] = {};
#pragma unroll
  for (int i = 0; i < NA; ++i)
#pragma unroll
    for (int j = 0; j < NB; ++j) Hab[i][j] = 0.5 * (at(Da, oa + i, ob + j) + at(Db, oa + i, ob + j));
#pragma unroll
  for (int k = 0; k < NC; ++k)
#pragma unroll
    for (int l = 0; l < ND; ++l) Hcd[k][l] = 0.5 * (at(Da, oc + k, od + l) + at(Db, oc + k, od + l));
#pragma unroll
  for (int i = 0; i < NA; ++i)
#pragma unroll
    for (int k = 0; k < NC; ++k) { Aac[i][k] = at(Da, oa + i, oc + k); Bac[i][k] = at(Db, oa + i, oc + k); }
#pragma unroll
  for (int j = 0; j < NB; ++j)
#pragma unroll
    for (int l = 0; l < ND; ++l) { Abd[j][l] = at(Da, ob + j, od + l); Bbd[j][l] = at(Db, ob + j, od + l); }
#pragma unroll
  for (int i = 0; i < NA; ++i)
#pragma unroll
    for (int l = 0; l < ND; ++l) { Aad[i][l] = at(Da, oa + i, od + l); Bad[i][l] = at(Db, oa + i, od + l); }
#pragma unroll
  for (int j = 0; j < NB; ++j)
#pragma unroll
    for (int k = 0; k < NC; ++k) { Abc[j][k] = at(Da, ob + j, oc + k); Bbc[j][k] = at(Db, ob + j, oc + k); }
#pragma unroll
  for (int i = 0; i < NA; ++i)
#pragma unroll
    for (int j = 0; j < NB; ++j)
#pragma unroll
      for (int k = 0; k < NC; ++k)
#pragma unroll
        for (int l = 0; l < ND; ++l) {
          const double v = deg * __ldg(store + (size_t)(((i * NB + j) * NC + k) * ND + l) * ntask + t);
          const double vq = -0.25 * v;
          gab[i][j] = fma(Hcd[k][l], v, gab[i][j]);
          gcd[k][l] = fma(Hab[i][j], v, gcd[k][l]);
          xac[i][k] = fma(Abd[j][l], vq, xac[i][k]); yac[i][k] = fma(Bbd[j][l], vq, yac[i][k]);
          xbd[j][l] = fma(Aac[i][k], vq, xbd[j][l]); ybd[j][l] = fma(Bac[i][k], vq, ybd[j][l]);
          xad[i][l] = fma(Abc[j][k], vq, xad[i][l]); yad[i][l] = fma(Bbc[j][k], vq, yad[i][l]);
          xbc[j][k] = fma(Aad[i][l], vq, xbc[j][k]); ybc[j][k] = fma(Bad[i][l], vq, ybc[j][k]);
        }
  auto add = [&](double* G, int i, int j, double v) { atomicAdd(G + (size_t)i * n + j, v); };
#pragma unroll
  for (int i = 0; i < NA; ++i)
#pragma unroll
    for (int j = 0; j < NB; ++j) add(GJ, oa + i, ob + j, gab[i][j]);
#pragma unroll
  for (int k = 0; k < NC; ++k)
#pragma unroll
    for (int l = 0; l < ND; ++l) add(GJ, oc + k, od + l, gcd[k][l]);
#pragma unroll
  for (int i = 0; i < NA; ++i)
#pragma unroll
    for (int k = 0; k < NC; ++k) { add(GKa, oa + i, oc + k, xac[i][k]); add(GKb, oa + i, oc + k, yac[i][k]); }
#pragma unroll
  for (int j = 0; j < NB; ++j)
#pragma unroll
    for (int l = 0; l < ND; ++l) { add(GKa, ob + j, od + l, xbd[j][l]); add(GKb, ob + j, od + l, ybd[j][l]); }
#pragma unroll
  for (int i = 0; i < NA; ++i)
#pragma unroll
    for (int l = 0; l < ND; ++l) { add(GKa, oa + i, od + l, xad[i][l]); add(GKb, oa + i, od + l, yad[i][l]); }
#pragma unroll
  for (int j = 0; j < NB; ++j)
#pragma unroll
    for (int k = 0; k < NC; ++k) { add(GKa, ob + j, oc + k, xbc[j][k]); add(GKb, ob + j, oc + k, ybc[j][k]); }
}

int pcg_launch_digest_u(int cls, const DevBasis& b, const DevPairsExt& pr, const int2* tasks, int ntask,
                        const double* store, const double* Da, const double* Db, double* GJ, double* GKa,
                        double* GKb, cudaStream_t s) {
  if (ntask <= 0) return PCG_OK;
  const int threads = 128, blocks = (ntask + threads - 1) / threads;
  switch (cls) {
#define X(id, a, bb, c, d) \
  case id: k_digest_u<a, bb, c, d><<<blocks, threads, 0, s>>>(b, pr, tasks, ntask, store, Da, Db, GJ, GKa, GKb); break;
    PCG_SHAPE_CASES(X)
#undef X
    default: return PCG_ERR_ARG;
  }
  PCG_CUDA(cudaGetLastError());
  return PCG_OK;
}


// Co-density digestion for non-orthogonal CI (the J and K of Methods/noci.py:243-300,
// hartree_fock.py:345-347 applied to non-symmetric densities): nd densities W (nd
// consecutive nbf x nbf blocks), one per blockIdx.y.  The accumulation is k_digest_u's
// with D_a = W and D_b = W^T: GJ_d receives the Coulomb part of (W + W^T)/2 and GK_d
// receives G[W^T] + G[W]^T (the D_a exchange blocks written transposed), so that
// J[W] = (GJ + GJ^T)/4 and K[W] = -GK/2 with K_ad = sum_bc (ab|cd) W_cb.
template <int NA, int NB, int NC, int ND>
__global__ void __launch_bounds__(128) k_digest_co(DevBasis b, DevPairsExt pr, const int2* __restrict__ tasks,
                                                   int ntask, const double* __restrict__ store,
                                                   const double* __restrict__ W, double* __restrict__ GJ,
                                                   double* __restrict__ GK, int d0) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntask) return;
  const int n = b.ld;
  const size_t dofs = (size_t)(d0 + blockIdx.y) * n * n;
  W += dofs; GJ += dofs; GK += dofs;
  const int2 tk = tasks[t];
  const int A = __ldg(pr.p.A + tk.x), B = __ldg(pr.p.B + tk.x);
  const int C = __ldg(pr.p.A + tk.y), Dd = __ldg(pr.p.B + tk.y);
  const int oa = __ldg(b.sh_ao + A), ob = __ldg(b.sh_ao + B), oc = __ldg(b.sh_ao + C), od = __ldg(b.sh_ao + Dd);
  const double deg = (A == B ? 1.0 : 2.0) * (C == Dd ? 1.0 : 2.0) * (tk.x == tk.y ? 1.0 : 2.0);
  auto w = [&](int i, int j) { return __ldg(W + (size_t)i * n + j); };
  double Hab[NA][NB], Hcd[NC][ND];
  double Aac[NA][NC], Abd[NB][ND], Aad[NA][ND], Abc[NB][NC];
  double Bac[NA][NC], Bbd[NB][ND], Bad[NA][ND], Bbc[NB][NC];
  double gab[NA][NB] = {}, gcd[NC][ND] = {};
  double xac[NA][NC] = {}, xbd[NB][ND] = {}, xad[NA][ND] = {}, xbc[NB][NC] = {};
  double yac[NA][NC] = {}, ybd[NB][ND] = {}, yad[NA][ND] = {}, ybc[NB][NC] = {};
#pragma unroll
  for (int i = 0; i < NA; ++i)
#pragma unroll
    for (int j = 0; j < NB; ++j) Hab[i][j] = 0.5 * (w(oa + i, ob + j) + w(ob + j, oa + i));
#pragma unroll
  for (int k = 0; k < NC; ++k)
#pragma unroll
    for (int l = 0; l < ND; ++l) Hcd[k][l] = 0.5 * (w(oc + k, od + l) + w(od + l, oc + k));
#pragma unroll
  for (int i = 0; i < NA; ++i)
#pragma unroll
    for (int k = 0; k < NC; ++k) { Aac[i][k] = w(oa + i, oc + k); Bac[i][k] = w(oc + k, oa + i); }
#pragma unroll
  for (int j = 0; j < NB; ++j)
#pragma unroll
    for (int l = 0; l < ND; ++l) { Abd[j][l] = w(ob + j, od + l); Bbd[j][l] = w(od + l, ob + j); }
#pragma unroll
  for (int i = 0; i < NA; ++i)
#pragma unroll
    for (int l = 0; l < ND; ++l) { Aad[i][l] = w(oa + i, od + l); Bad[i][l] = w(od + l, oa + i); }
#pragma unroll
  for (int j = 0; j < NB; ++j)
#pragma unroll
    for (int k = 0; k < NC; ++k) { Abc[j][k] = w(ob + j, oc + k); Bbc[j][k] = w(oc + k, ob + j); }
#pragma unroll
  for (int i = 0; i < NA; ++i)
#pragma unroll
    for (int j = 0; j < NB; ++j)
#pragma unroll
      for (int k = 0; k < NC; ++k)
#pragma unroll
        for (int l = 0; l < ND; ++l) {
          const double v = deg * __ldg(store + (size_t)(((i * NB + j) * NC + k) * ND + l) * ntask + t);
          const double vq = -0.25 * v;
          gab[i][j] = fma(Hcd[k][l], v, gab[i][j]);
          gcd[k][l] = fma(Hab[i][j], v, gcd[k][l]);
          xac[i][k] = fma(Abd[j][l], vq, xac[i][k]); yac[i][k] = fma(Bbd[j][l], vq, yac[i][k]);
          xbd[j][l] = fma(Aac[i][k], vq, xbd[j][l]); ybd[j][l] = fma(Bac[i][k], vq, ybd[j][l]);
          xad[i][l] = fma(Abc[j][k], vq, xad[i][l]); yad[i][l] = fma(Bbc[j][k], vq, yad[i][l]);
          xbc[j][k] = fma(Aad[i][l], vq, xbc[j][k]); ybc[j][k] = fma(Bad[i][l], vq, ybc[j][k]);
        }
  auto add = [&](double* G, int i, int j, double v) { atomicAdd(G + (size_t)i * n + j, v); };
#pragma unroll
  for (int i = 0; i < NA; ++i)
#pragma unroll
    for (int j = 0; j < NB; ++j) add(GJ, oa + i, ob + j, gab[i][j]);
#pragma unroll
  for (int k = 0; k < NC; ++k)
#pragma unroll
    for (int l = 0; l < ND; ++l) add(GJ, oc + k, od + l, gcd[k][l]);
  // x: G[W] (written transposed), y: G[W^T]
#pragma unroll
  for (int i = 0; i < NA; ++i)
#pragma unroll
    for (int k = 0; k < NC; ++k) { add(GK, oc + k, oa + i, xac[i][k]); add(GK, oa + i, oc + k, yac[i][k]); }
#pragma unroll
  for (int j = 0; j < NB; ++j)
#pragma unroll
    for (int l = 0; l < ND; ++l) { add(GK, od + l, ob + j, xbd[j][l]); add(GK, ob + j, od + l, ybd[j][l]); }
#pragma unroll
  for (int i = 0; i < NA; ++i)
#pragma unroll
    for (int l = 0; l < ND; ++l) { add(GK, od + l, oa + i, xad[i][l]); add(GK, oa + i, od + l, yad[i][l]); }
#pragma unroll
  for (int j = 0; j < NB; ++j)
#pragma unroll
    for (int k = 0; k < NC; ++k) { add(GK, oc + k, ob + j, xbc[j][k]); add(GK, ob + j, oc + k, ybc[j][k]); }
}

int pcg_launch_digest_co(int cls, const DevBasis& b, const DevPairsExt& pr, const int2* tasks, int ntask,
                         const double* store, int nd, const double* W, double* GJ, double* GK, cudaStream_t s) {
  if (ntask <= 0 || nd <= 0) return PCG_OK;
  const int threads = 128, blocks = (ntask + threads - 1) / threads;
  for (int d0 = 0; d0 < nd; d0 += 65535) {
    const dim3 grid(blocks, nd - d0 < 65535 ? nd - d0 : 65535);
    switch (cls) {
#define X(id, a, bb, c, d) \
  case id: k_digest_co<a, bb, c, d><<<grid, threads, 0, s>>>(b, pr, tasks, ntask, store, W, GJ, GK, d0); break;
      PCG_SHAPE_CASES(X)
#undef X
      default: return PCG_ERR_ARG;
    }
    PCG_CUDA(cudaGetLastError());
  }
  return PCG_OK;
}
