// Electron-repulsion integrals over Schwarz-screened shell quartets, Fock digestion
// and dense expansion.
//
// Upstream counterparts: Methods/integrals.py:427-555 (two_electron: fundamentals,
// VRR, contraction, HRR, normalisation, spherical transform),
// Methods/c_ints/two_electron_{fundamentals,vrr,contract,hrr}.c, the screened quartet
// loop and 8-fold store of Methods/hartree_fock.py:241-325, and the J/K contraction
// of Methods/hartree_fock.py:329-355.
//
// Layout: one task = one canonical shell quartet (bra pair, ket pair) of a class;
// tasks of a class are grouped in buckets of equal primitive counts so a warp runs
// uniform loops.  Results of a class are stored class-major
//     store[k * ntask + t]   (k = spherical element, t = task)
// so writes here and reads in the digestion are coalesced across a warp.
#include "common.cuh"
#include "pcg_internal.h"

// ----------------------------------------------------------------------------------
// Fock digestion (closed shell): for every stored quartet block, with the shell-level
// degeneracy d = (A!=B ? 2:1)(C!=D ? 2:1)(AB!=CD ? 2:1) and v' = d (ab|cd),
//   G_ab += D_cd v', G_cd += D_ab v', G_ac -= D_bd v'/4, G_bd -= D_ac v'/4,
//   G_ad -= D_bc v'/4, G_bc -= D_ad v'/4;
// the caller symmetrises F = H + (G + G^T)/2, which equals H + 2J[D] - K[D] with D the
// alpha density -- upstream's H + J[D_a + D_b] - K[D_a] (hartree_fock.py:345-355).
// ----------------------------------------------------------------------------------
template <int NA, int NB, int NC, int ND>
__global__ void __launch_bounds__(128) k_digest(DevBasis b, DevPairsExt pr, const int2* __restrict__ tasks,
                                                int ntask, const double* __restrict__ store,
                                                const double* __restrict__ D, double* __restrict__ G) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntask) return;
  const int2 tk = tasks[t];
  int oa, ob, oc, od;
  long long o;  // the four shells share one molecule block
  bool sab, scd;
  if (pr.p.ao4) {  // one 16-byte load per pair instead of the shell tables
    const int4 pb = __ldg(pr.p.ao4 + tk.x), pk = __ldg(pr.p.ao4 + tk.y);
    oa = pb.x & 0x3FFFFFFF; ob = pb.y; oc = pk.x & 0x3FFFFFFF; od = pk.y;
    sab = (pb.x >> 30) & 1; scd = (pk.x >> 30) & 1;
    o = (long long)(unsigned)pb.z | ((long long)pb.w << 32);
  } else {
    const int A = __ldg(pr.p.A + tk.x), B = __ldg(pr.p.B + tk.x);
    const int C = __ldg(pr.p.A + tk.y), Dd = __ldg(pr.p.B + tk.y);
    o = dev_blk(b, A);
    oa = __ldg(b.sh_ao + A); ob = __ldg(b.sh_ao + B); oc = __ldg(b.sh_ao + C); od = __ldg(b.sh_ao + Dd);
    sab = A == B; scd = C == Dd;
  }
  const int n = b.ld;
  D += o;
  G += o;
  const double deg = (sab ? 1.0 : 2.0) * (scd ? 1.0 : 2.0) * (tk.x == tk.y ? 1.0 : 2.0);
  double Dab[NA][NB], Dcd[NC][ND], Dac[NA][NC], Dbd[NB][ND], Dad[NA][ND], Dbc[NB][NC];
  double gab[NA][NB], gcd[NC][ND], gac[NA][NC], gbd[NB][ND], gad[NA][ND], gbc[NB][NC];
#pragma unroll
  for (int i = 0; i < NA; ++i)
#pragma unroll
    for (int j = 0; j < NB; ++j) { Dab[i][j] = __ldg(D + (size_t)(oa + i) * n + ob + j); gab[i][j] = 0.0; }
#pragma unroll
  for (int k = 0; k < NC; ++k)
#pragma unroll
    for (int l = 0; l < ND; ++l) { Dcd[k][l] = __ldg(D + (size_t)(oc + k) * n + od + l); gcd[k][l] = 0.0; }
#pragma unroll
  for (int i = 0; i < NA; ++i)
#pragma unroll
    for (int k = 0; k < NC; ++k) { Dac[i][k] = __ldg(D + (size_t)(oa + i) * n + oc + k); gac[i][k] = 0.0; }
#pragma unroll
  for (int j = 0; j < NB; ++j)
#pragma unroll
    for (int l = 0; l < ND; ++l) { Dbd[j][l] = __ldg(D + (size_t)(ob + j) * n + od + l); gbd[j][l] = 0.0; }
#pragma unroll
  for (int i = 0; i < NA; ++i)
#pragma unroll
    for (int l = 0; l < ND; ++l) { Dad[i][l] = __ldg(D + (size_t)(oa + i) * n + od + l); gad[i][l] = 0.0; }
#pragma unroll
  for (int j = 0; j < NB; ++j)
#pragma unroll
    for (int k = 0; k < NC; ++k) { Dbc[j][k] = __ldg(D + (size_t)(ob + j) * n + oc + k); gbc[j][k] = 0.0; }
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
          gab[i][j] = fma(Dcd[k][l], v, gab[i][j]);
          gcd[k][l] = fma(Dab[i][j], v, gcd[k][l]);
          gac[i][k] = fma(Dbd[j][l], vq, gac[i][k]);
          gbd[j][l] = fma(Dac[i][k], vq, gbd[j][l]);
          gad[i][l] = fma(Dbc[j][k], vq, gad[i][l]);
          gbc[j][k] = fma(Dad[i][l], vq, gbc[j][k]);
        }
#pragma unroll
  for (int i = 0; i < NA; ++i)
#pragma unroll
    for (int j = 0; j < NB; ++j) atomicAdd(G + (size_t)(oa + i) * n + ob + j, gab[i][j]);
#pragma unroll
  for (int k = 0; k < NC; ++k)
#pragma unroll
    for (int l = 0; l < ND; ++l) atomicAdd(G + (size_t)(oc + k) * n + od + l, gcd[k][l]);
#pragma unroll
  for (int i = 0; i < NA; ++i)
#pragma unroll
    for (int k = 0; k < NC; ++k) atomicAdd(G + (size_t)(oa + i) * n + oc + k, gac[i][k]);
#pragma unroll
  for (int j = 0; j < NB; ++j)
#pragma unroll
    for (int l = 0; l < ND; ++l) atomicAdd(G + (size_t)(ob + j) * n + od + l, gbd[j][l]);
#pragma unroll
  for (int i = 0; i < NA; ++i)
#pragma unroll
    for (int l = 0; l < ND; ++l) atomicAdd(G + (size_t)(oa + i) * n + od + l, gad[i][l]);
#pragma unroll
  for (int j = 0; j < NB; ++j)
#pragma unroll
    for (int k = 0; k < NC; ++k) atomicAdd(G + (size_t)(ob + j) * n + oc + k, gbc[j][k]);
}

// Dense N^4 store with the 8-fold permutational symmetry (hartree_fock.py:314-325).
template <int NA, int NB, int NC, int ND>
__global__ void k_dense(DevBasis b, DevPairsExt pr, const int2* __restrict__ tasks, int ntask,
                        const double* __restrict__ store, double* __restrict__ eri) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntask) return;
  const int2 tk = tasks[t];
  const int oa = b.sh_ao[pr.p.A[tk.x]], ob = b.sh_ao[pr.p.B[tk.x]];
  const int oc = b.sh_ao[pr.p.A[tk.y]], od = b.sh_ao[pr.p.B[tk.y]];
  const size_t n = b.nbf;
  for (int i = 0; i < NA; ++i)
    for (int j = 0; j < NB; ++j)
      for (int k = 0; k < NC; ++k)
        for (int l = 0; l < ND; ++l) {
          const double v = store[(size_t)(((i * NB + j) * NC + k) * ND + l) * ntask + t];
          const size_t a = oa + i, bb = ob + j, c = oc + k, d = od + l;
          eri[((a * n + bb) * n + c) * n + d] = v;
          eri[((bb * n + a) * n + c) * n + d] = v;
          eri[((a * n + bb) * n + d) * n + c] = v;
          eri[((bb * n + a) * n + d) * n + c] = v;
          eri[((c * n + d) * n + a) * n + bb] = v;
          eri[((d * n + c) * n + a) * n + bb] = v;
          eri[((c * n + d) * n + bb) * n + a] = v;
          eri[((d * n + c) * n + bb) * n + a] = v;
        }
}

// The dense tensor with the bra pair packed, E[pair(a, b)][c][d] for a >= b (pair(a, b)
// = a(a+1)/2 + b): half of the N^4 tensor, the input of the first MP2 transform, which
// keeps the bra symmetry; each stored element goes to its four images with a >= b.
__device__ __forceinline__ size_t ao_pair(size_t a, size_t b) { return a >= b ? a * (a + 1) / 2 + b : b * (b + 1) / 2 + a; }

template <int NA, int NB, int NC, int ND>
__global__ void k_dense_pairs(DevBasis b, DevPairsExt pr, const int2* __restrict__ tasks, int ntask,
                              const double* __restrict__ store, const int* __restrict__ pmap,
                              double* __restrict__ E) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntask) return;
  const int2 tk = tasks[t];
  const int oa = b.sh_ao[pr.p.A[tk.x]], ob = b.sh_ao[pr.p.B[tk.x]];
  const int oc = b.sh_ao[pr.p.A[tk.y]], od = b.sh_ao[pr.p.B[tk.y]];
  const size_t n = b.nbf;
  for (int i = 0; i < NA; ++i)
    for (int j = 0; j < NB; ++j) {
      const long long pab = pmap ? (long long)__ldg(pmap + ao_pair(oa + i, ob + j)) : (long long)ao_pair(oa + i, ob + j);
      for (int k = 0; k < NC; ++k)
        for (int l = 0; l < ND; ++l) {
          const double v = store[(size_t)(((i * NB + j) * NC + k) * ND + l) * ntask + t];
          const size_t a = oa + i, bb = ob + j, c = oc + k, d = od + l;
          const long long pcd = pmap ? (long long)__ldg(pmap + ao_pair(c, d)) : (long long)ao_pair(c, d);
          // a pair without a row (map -1) is written nowhere
          if (pab >= 0) {
            E[((size_t)pab * n + c) * n + d] = v;
            E[((size_t)pab * n + d) * n + c] = v;
          }
          if (pcd >= 0) {
            E[((size_t)pcd * n + a) * n + bb] = v;
            E[((size_t)pcd * n + bb) * n + a] = v;
          }
        }
    }
}

// The symmetric pair matrix of the compact rows: M[map(pair(a, b))][map(pair(c, d))] =
// (ab|cd) for the AO pairs with rows (rows x rows, both triangles written); an element
// whose bra or ket pair has no row belongs to the diagonal quartet of such a pair and
// is left out with it.  Two stores per stored element instead of four.
template <int NA, int NB, int NC, int ND>
__global__ void k_sym_pairs(DevBasis b, DevPairsExt pr, const int2* __restrict__ tasks, int ntask,
                            const double* __restrict__ store, const int* __restrict__ pmap, long long rows,
                            double* __restrict__ M) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntask) return;
  const int2 tk = tasks[t];
  const int oa = b.sh_ao[pr.p.A[tk.x]], ob = b.sh_ao[pr.p.B[tk.x]];
  const int oc = b.sh_ao[pr.p.A[tk.y]], od = b.sh_ao[pr.p.B[tk.y]];
  int pcd[NC * ND];
#pragma unroll
  for (int k = 0; k < NC; ++k)
#pragma unroll
    for (int l = 0; l < ND; ++l) pcd[k * ND + l] = __ldg(pmap + ao_pair(oc + k, od + l));
  for (int i = 0; i < NA; ++i)
    for (int j = 0; j < NB; ++j) {
      const int pab = __ldg(pmap + ao_pair(oa + i, ob + j));
      if (pab < 0) continue;
#pragma unroll
      for (int kl = 0; kl < NC * ND; ++kl) {
        if (pcd[kl] < 0) continue;
        const double v = store[(size_t)((i * NB + j) * NC * ND + kl) * ntask + t];
        M[(size_t)pab * rows + pcd[kl]] = v;
        M[(size_t)pcd[kl] * rows + pab] = v;
      }
    }
}

// used[p] = 1 for both pairs of every task (x, y) with x != y; a byte is read before it
// is written, so the many tasks of one pair store it once or a few times
__global__ void k_mark_pairs(const int2* __restrict__ tasks, int ntask, unsigned char* __restrict__ used) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntask) return;
  const int2 tk = tasks[t];
  if (tk.x == tk.y) return;
  if (!used[tk.x]) used[tk.x] = 1;
  if (!used[tk.y]) used[tk.y] = 1;
}

// colmap[a*n + b] = pmap[pair(a, b)] (pair(a, b) itself without pmap): where each
// (a, b) of an unpacked row is found in a pair-packed row, -1 for none
__global__ void k_pair_colmap(int n, const int* __restrict__ pmap, int* __restrict__ colmap) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n * n) return;
  const int a = idx / n, bb = idx - a * n;
  const size_t p = ao_pair(a, bb);
  colmap[idx] = pmap ? pmap[p] : (int)p;
}

// out[r][ab] = in[r][colmap[ab]] (0 where colmap is -1), one block per row (grid-
// stride over rows); with SH the packed row is staged in shared memory first, so the
// gather reads shared memory and both global streams are coalesced
template <bool SH>
__global__ void __launch_bounds__(512) k_unpack_rows(long long R, int nn, int len, const int* __restrict__ colmap,
                                                      const double* __restrict__ in, double* __restrict__ out) {
  extern __shared__ double row_sh[];
  for (long long r = blockIdx.x; r < R; r += gridDim.x) {
    const double* src = in + r * len;
    if (SH) {
      __syncthreads();
      for (int q = threadIdx.x; q < len; q += blockDim.x) row_sh[q] = __ldcs(src + q);
      __syncthreads();
    }
    double* dst = out + r * nn;
    if (SH && (nn & 1) == 0) {
      // two elements per thread: one 8-byte map load and one 16-byte store (rows of an
      // even length keep the output 16-byte aligned)
      const int2* cm2 = (const int2*)colmap;
      double2* d2 = (double2*)dst;
      for (int h = threadIdx.x; h < nn / 2; h += blockDim.x) {
        const int2 q = __ldg(cm2 + h);
        __stcs(d2 + h, make_double2(q.x < 0 ? 0.0 : row_sh[q.x], q.y < 0 ? 0.0 : row_sh[q.y]));
      }
    } else {
      for (int ab = threadIdx.x; ab < nn; ab += blockDim.x) {
        const int q = __ldg(colmap + ab);
        __stcs(dst + ab, q < 0 ? 0.0 : (SH ? row_sh[q] : __ldg(src + q)));
      }
    }
  }
}

int pcg_launch_dense_pairs(int cls, const DevBasis& b, const DevPairsExt& pr, const int2* tasks, int ntask,
                           const double* store, const int* pmap, double* E, cudaStream_t s) {
  if (ntask <= 0) return PCG_OK;
  const int threads = 128, blocks = (ntask + threads - 1) / threads;
  switch (cls) {
#define X(id, a, bb, c, d) \
  case id: k_dense_pairs<a, bb, c, d><<<blocks, threads, 0, s>>>(b, pr, tasks, ntask, store, pmap, E); break;
    PCG_SHAPE_CASES(X)
#undef X
    default: pcg_set_error("pcg_dense_pairs_class: class id out of range"); return PCG_ERR_ARG;
  }
  PCG_CUDA(cudaGetLastError());
  return PCG_OK;
}

int pcg_launch_sym_pairs(int cls, const DevBasis& b, const DevPairsExt& pr, const int2* tasks, int ntask,
                         const double* store, const int* pmap, long long rows, double* M, cudaStream_t s) {
  if (ntask <= 0) return PCG_OK;
  const int threads = 128, blocks = (ntask + threads - 1) / threads;
  switch (cls) {
#define X(id, a, bb, c, d) \
  case id: k_sym_pairs<a, bb, c, d><<<blocks, threads, 0, s>>>(b, pr, tasks, ntask, store, pmap, rows, M); break;
    PCG_SHAPE_CASES(X)
#undef X
    default: pcg_set_error("pcg_sym_pairs_class: class id out of range"); return PCG_ERR_ARG;
  }
  PCG_CUDA(cudaGetLastError());
  return PCG_OK;
}

int pcg_launch_mark_pairs(const int2* tasks, int ntask, unsigned char* used, cudaStream_t s) {
  if (ntask <= 0) return PCG_OK;
  k_mark_pairs<<<(ntask + 255) / 256, 256, 0, s>>>(tasks, ntask, used);
  PCG_CUDA(cudaGetLastError());
  return PCG_OK;
}

int pcg_launch_pair_colmap(int n, const int* pmap, int* colmap, cudaStream_t s) {
  k_pair_colmap<<<(n * n + 255) / 256, 256, 0, s>>>(n, pmap, colmap);
  PCG_CUDA(cudaGetLastError());
  return PCG_OK;
}

int pcg_launch_unpack_rows(long long R, int n, int len, const int* colmap, const double* in, double* out,
                           cudaStream_t s) {
  if (R <= 0) return PCG_OK;
  const unsigned blocks = (unsigned)(R < 152LL * 64 ? R : 152LL * 64);
  const size_t sh = (size_t)len * sizeof(double);
  if (sh <= 100 * 1024) {
    PCG_CUDA(cudaFuncSetAttribute(k_unpack_rows<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024));
    k_unpack_rows<true><<<blocks, 512, sh, s>>>(R, n * n, len, colmap, in, out);
  } else {
    k_unpack_rows<false><<<blocks, 512, 0, s>>>(R, n * n, len, colmap, in, out);
  }
  PCG_CUDA(cudaGetLastError());
  return PCG_OK;
}

// Schwarz factor per shell pair from its diagonal block (ab|ab): sqrt(max (mn|mn)),
// the upstream bound of hartree_fock.py:244-254 reduced to the pair level.
template <int NA, int NB>
__global__ void k_schwarz(const int2* __restrict__ tasks, int ntask, const double* __restrict__ store,
                          double* __restrict__ Q) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntask) return;
  double m = 0.0;
  for (int i = 0; i < NA; ++i)
    for (int j = 0; j < NB; ++j) {
      const double v = store[(size_t)(((i * NB + j) * NA + i) * NB + j) * ntask + t];
      m = fmax(m, v);
    }
  Q[tasks[t].x] = sqrt(m);
}

// ----------------------------------------------------------------------------------
// Class table and dispatch
// ----------------------------------------------------------------------------------
static const int kClassL[21][4] = {
    {0, 0, 0, 0}, {1, 0, 0, 0}, {1, 0, 1, 0}, {1, 1, 0, 0}, {1, 1, 1, 0}, {1, 1, 1, 1}, {2, 0, 0, 0},
    {2, 0, 1, 0}, {2, 0, 1, 1}, {2, 0, 2, 0}, {2, 1, 0, 0}, {2, 1, 1, 0}, {2, 1, 1, 1}, {2, 1, 2, 0},
    {2, 1, 2, 1}, {2, 2, 0, 0}, {2, 2, 1, 0}, {2, 2, 1, 1}, {2, 2, 2, 0}, {2, 2, 2, 1}, {2, 2, 2, 2}};

static int pair_class(int la, int lb) { return la * (la + 1) / 2 + lb; }

int pcg_class_id(int la, int lb, int lc, int ld) {
  if (la < lb || lc < ld || la > PCG_MAXL || lc > PCG_MAXL) return -1;
  int pb = pair_class(la, lb), pk = pair_class(lc, ld);
  if (pb < pk) return -1;
  return pb * (pb + 1) / 2 + pk;
}

int pcg_class_nout(int cls) {
  if (cls < 0 || cls >= 21) return 0;
  const int* l = kClassL[cls];
  return (2 * l[0] + 1) * (2 * l[1] + 1) * (2 * l[2] + 1) * (2 * l[3] + 1);
}

int pcg_launch_eri_g0(int, const DevPairsExt&, const BoysTable&, const int2*, int, double*, int, cudaStream_t);
int pcg_launch_eri_g1(int, const DevPairsExt&, const BoysTable&, const int2*, int, double*, int, cudaStream_t);
int pcg_launch_eri_g2(int, const DevPairsExt&, const BoysTable&, const int2*, int, double*, int, cudaStream_t);
int pcg_launch_eri_g3(int, const DevPairsExt&, const BoysTable&, const int2*, int, double*, int, cudaStream_t);
int pcg_launch_eri_g4(int, const DevPairsExt&, const BoysTable&, const int2*, int, double*, int, cudaStream_t);
int pcg_launch_eri_g5(int, const DevPairsExt&, const BoysTable&, const int2*, int, double*, int, cudaStream_t);

int pcg_launch_eri(int cls, const DevBasis& b, const DevPairsExt& pr, const BoysTable& bt, const int2* tasks,
                   int ntask, double* store, int precision, float, const double*, cudaStream_t s) {
  (void)b;
  if (ntask <= 0) return PCG_OK;
  if (cls < 0 || cls > 20) return PCG_ERR_ARG;
  if (cls <= 5) return pcg_launch_eri_g0(cls, pr, bt, tasks, ntask, store, precision, s);
  if (cls <= 13) return pcg_launch_eri_g1(cls, pr, bt, tasks, ntask, store, precision, s);
  if (cls <= 17) return pcg_launch_eri_g2(cls, pr, bt, tasks, ntask, store, precision, s);
  if (cls <= 19) return pcg_launch_eri_g3(cls, pr, bt, tasks, ntask, store, precision, s);
  if (precision == 0) return pcg_launch_eri_g4(cls, pr, bt, tasks, ntask, store, precision, s);
  return pcg_launch_eri_g5(cls, pr, bt, tasks, ntask, store, precision, s);
}

int pcg_launch_scattering(int cls, const DevPairsExt& pr, const int2* tasks, int ntask, double S, double* store,
                          cudaStream_t s) {
  if (ntask <= 0) return PCG_OK;
  if (cls < 0 || cls > 20) return PCG_ERR_ARG;
  if (cls <= 13) return pcg_launch_eri_s0(cls, pr, tasks, ntask, S, store, s);
  if (cls <= 17) return pcg_launch_eri_s1(cls, pr, tasks, ntask, S, store, s);
  if (cls <= 19) return pcg_launch_eri_s2(cls, pr, tasks, ntask, S, store, s);
  return pcg_launch_eri_s3(cls, pr, tasks, ntask, S, store, s);
}

int pcg_launch_digest(int cls, const DevBasis& b, const DevPairsExt& pr, const int2* tasks, int ntask,
                      const double* store, const double* D, double* G, cudaStream_t s) {
  if (ntask <= 0) return PCG_OK;
  const int threads = 128, blocks = (ntask + threads - 1) / threads;
  switch (cls) {
#define X(id, a, bb, c, d) \
  case id: k_digest<a, bb, c, d><<<blocks, threads, 0, s>>>(b, pr, tasks, ntask, store, D, G); break;
    PCG_SHAPE_CASES(X)
#undef X
    default: pcg_set_error("pcg_digest_class: class id out of range"); return PCG_ERR_ARG;
  }
  PCG_CUDA(cudaGetLastError());
  return PCG_OK;
}

int pcg_launch_dense(int cls, const DevBasis& b, const DevPairsExt& pr, const int2* tasks, int ntask,
                     const double* store, double* eri, cudaStream_t s) {
  if (ntask <= 0) return PCG_OK;
  const int threads = 128, blocks = (ntask + threads - 1) / threads;
  switch (cls) {
#define X(id, a, bb, c, d) \
  case id: k_dense<a, bb, c, d><<<blocks, threads, 0, s>>>(b, pr, tasks, ntask, store, eri); break;
    PCG_SHAPE_CASES(X)
#undef X
    default: return PCG_ERR_ARG;
  }
  PCG_CUDA(cudaGetLastError());
  return PCG_OK;
}

int pcg_launch_schwarz(int cls, const int2* tasks, int ntask, const double* store, double* Q, cudaStream_t s) {
  if (ntask <= 0) return PCG_OK;
  const int threads = 128, blocks = (ntask + threads - 1) / threads;
  switch (cls) {
    case 0: k_schwarz<1, 1><<<blocks, threads, 0, s>>>(tasks, ntask, store, Q); break;
    case 2: k_schwarz<3, 1><<<blocks, threads, 0, s>>>(tasks, ntask, store, Q); break;
    case 5: k_schwarz<3, 3><<<blocks, threads, 0, s>>>(tasks, ntask, store, Q); break;
    case 9: k_schwarz<5, 1><<<blocks, threads, 0, s>>>(tasks, ntask, store, Q); break;
    case 14: k_schwarz<5, 3><<<blocks, threads, 0, s>>>(tasks, ntask, store, Q); break;
    case 20: k_schwarz<5, 5><<<blocks, threads, 0, s>>>(tasks, ntask, store, Q); break;
    default: return PCG_ERR_ARG;
  }
  PCG_CUDA(cudaGetLastError());
  return PCG_OK;
}

// ----------------------------------------------------------------------------------
// Task expansion: row r pairs bra pair bra[r] with the kets at positions
// [qstart[r], qstart[r] + cnt[r] - diag[r]) of the ket list, plus the bra's own pair
// when diag[r] (the diagonal quartet upstream always computes); cnt[r] = off[r+1] -
// off[r].
// ----------------------------------------------------------------------------------
__global__ void k_expand(int nbra, const int* __restrict__ bra, const int* __restrict__ ket,
                         const long long* __restrict__ off, const int* __restrict__ qstart,
                         const int* __restrict__ diag, long long ntask, int2* __restrict__ out) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntask) return;
  int lo = 0, hi = nbra - 1;  // last r with off[r] <= t
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (off[mid] <= t) lo = mid; else hi = mid - 1;
  }
  const int r = lo;
  const long long q = t - off[r];
  const long long cnt = off[r + 1] - off[r];
  int kp;
  if (diag[r] && q == cnt - 1) kp = bra[r];
  else kp = ket[qstart[r] + q];
  out[t] = make_int2(bra[r], kp);
}

int pcg_launch_expand(int nbra, const int* bra, const int* ket, const long long* off, const int* qstart,
                      const int* diag, long long ntask, int2* out, cudaStream_t s) {
  if (ntask <= 0) return PCG_OK;
  const int threads = 256;
  const long long blocks = (ntask + threads - 1) / threads;
  k_expand<<<(unsigned)blocks, threads, 0, s>>>(nbra, bra, ket, off, qstart, diag, ntask, out);
  PCG_CUDA(cudaGetLastError());
  return PCG_OK;
}

// F = H + (G + G^T) / 2
__global__ void k_fock(int n, const double* __restrict__ H, const double* __restrict__ G, double* __restrict__ F) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n * n) return;
  const int i = idx / n, j = idx % n;
  F[idx] = H[idx] + 0.5 * (G[idx] + G[(size_t)j * n + i]);
}

// F = H + (G + G^T)/2 for nblocks consecutive ld x ld blocks
__global__ void k_fock_batched(long long total, int ld, const double* __restrict__ H, const double* __restrict__ G,
                               double* __restrict__ F) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= total) return;
  const long long sq = (long long)ld * ld;
  const long long base = idx / sq * sq;
  const int r = (int)(idx - base);
  const int i = r / ld, j = r % ld;
  F[idx] = H[idx] + 0.5 * (G[idx] + G[base + (long long)j * ld + i]);
}

int pcg_launch_fock_batched(int nblocks, int ld, const double* H, const double* G, double* F, cudaStream_t s) {
  const long long total = (long long)nblocks * ld * ld;
  k_fock_batched<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(total, ld, H, G, F);
  PCG_CUDA(cudaGetLastError());
  return PCG_OK;
}

int pcg_launch_fock(int n, const double* H, const double* G, double* F, cudaStream_t s) {
  if (n <= 0) return PCG_OK;
  k_fock<<<(n * n + 255) / 256, 256, 0, s>>>(n, H, G, F);
  PCG_CUDA(cudaGetLastError());
  return PCG_OK;
}
