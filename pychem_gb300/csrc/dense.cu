// Small dense FP64 algebra of the SCF iteration, all on the GPU:
//
//  * pcg_dgemm: batched C = alpha A B + beta C with arbitrary element strides (so any
//    transposes), 8 x 8 output tiles of one thread per element.  GB300's FP64 pipe
//    is thin (about 1.7 FMA per clock per SM), so the SCF's n <= 300 products are
//    spread over many CTAs: 676 for n = 208.  Replaces the numpy.dot /
//    matrix products of Methods/hartree_fock.py:168-184 and
//    Methods/hf_extensions/diis.py:48-54 (X^T F X, the commutator, C = X C').
//  * pcg_oa_correction: the correction matrix of one Ogita-Aishima refinement step of
//    approximate eigenvectors (T. Ogita, K. Aishima, Japan J. Indust. Appl. Math. 35
//    (2018) 1007-1035, Algorithm 1) from S = X^T A X and R = I - X^T X.
//  * DIIS (Methods/hf_extensions/diis.py:32-41,108-112): Fock matrices and residuals
//    in a ring of `cap` slots, the new row of the residual inner-product matrix, the
//    C1 system solved by one CTA (Gaussian elimination with partial pivoting, the
//    oldest vectors dropped while it is singular), and the extrapolation -- no host
//    round trip, so an SCF iteration can be captured in a CUDA graph.
#include <math.h>

#include "../../include/pychem_gb300.h"
#include "common.cuh"
#include "pcg_internal.h"

// 8 x 8 output tiles (one thread per element), K in steps of 32: at n = 208 that is
// 676 CTAs, 4-5 per SM, so the FP64 work is spread evenly over the 152 SMs (with
// 16 x 16 tiles the 169 CTAs left 17 SMs with twice the work of the others).
#define DG_T 8
#define DG_K 32

__global__ void __launch_bounds__(DG_T* DG_T)
    k_dgemm(int M, int N, int K, double alpha, const double* __restrict__ A, long long sAb, long long sAm,
            long long sAk, const double* __restrict__ B, long long sBb, long long sBk, long long sBn, double beta,
            double* __restrict__ C, long long sCb, long long sCm, long long sCn) {
  // two shared-memory stages: the next K step's tile is loaded into registers while
  // the current one is multiplied, so the global-load latency overlaps the FMAs
  __shared__ double As[2][DG_T][DG_K + 1], Bs[2][DG_K][DG_T + 1];
  constexpr int PER = DG_T * DG_K / (DG_T * DG_T);   // elements of each tile per thread
  const int tid = threadIdx.x, tx = tid % DG_T, ty = tid / DG_T;
  const long long b = blockIdx.z;
  const int m0 = blockIdx.y * DG_T, n0 = blockIdx.x * DG_T;
  const int m = m0 + ty, n = n0 + tx;
  A += b * sAb;
  B += b * sBb;
  double ra[PER], rb[PER];
  auto load = [&](int k0) {
#pragma unroll
    for (int u = 0; u < PER; ++u) {
      const int e = tid + u * DG_T * DG_T;
      const int mr = m0 + e / DG_K, ka = k0 + e % DG_K;
      ra[u] = (mr < M && ka < K) ? __ldg(A + mr * sAm + ka * sAk) : 0.0;
      const int kb = k0 + e / DG_T, c = n0 + e % DG_T;
      rb[u] = (kb < K && c < N) ? __ldg(B + kb * sBk + c * sBn) : 0.0;
    }
  };
  auto store = [&](int st) {
#pragma unroll
    for (int u = 0; u < PER; ++u) {
      const int e = tid + u * DG_T * DG_T;
      As[st][e / DG_K][e % DG_K] = ra[u];
      Bs[st][e / DG_T][e % DG_T] = rb[u];
    }
  };
  double acc = 0.0;
  load(0);
  store(0);
  __syncthreads();
  int st = 0;
  for (int k0 = 0; k0 < K; k0 += DG_K) {
    const bool more = k0 + DG_K < K;
    if (more) load(k0 + DG_K);
#pragma unroll
    for (int kk = 0; kk < DG_K; ++kk) acc = fma(As[st][ty][kk], Bs[st][kk][tx], acc);
    if (more) store(st ^ 1);
    __syncthreads();
    st ^= 1;
  }
  if (m < M && n < N) {
    double* c = C + b * sCb + m * sCm + n * sCn;
    *c = beta == 0.0 ? alpha * acc : fma(alpha, acc, beta * *c);
  }
}

extern "C" int pcg_dgemm(int batch, int M, int N, int K, double alpha, const double* A, long long sAb, long long sAm,
                         long long sAk, const double* B, long long sBb, long long sBk, long long sBn, double beta,
                         double* C, long long sCb, long long sCm, long long sCn, void* stream) {
  if (batch < 1 || M < 0 || N < 0 || K < 0 || batch > 65535 || (M > 0 && N > 0 && (!C || (K > 0 && (!A || !B))))) {
    pcg_set_error("pcg_dgemm: bad arguments");
    return PCG_ERR_ARG;
  }
  if (M == 0 || N == 0) return PCG_OK;
  dim3 grid((N + DG_T - 1) / DG_T, (M + DG_T - 1) / DG_T, batch);
  if (grid.y > 65535) { pcg_set_error("pcg_dgemm: M too large"); return PCG_ERR_UNSUPPORTED; }
  k_dgemm<<<grid, DG_T * DG_T, 0, (cudaStream_t)stream>>>(M, N, K, alpha, A, sAb, sAm, sAk, B, sBb, sBk, sBn, beta,
                                                          C, sCb, sCm, sCn);
  PCG_CUDA(cudaGetLastError());
  return PCG_OK;
}

// E[i][j] for one refinement step X <- X + X E, with lam_i = S_ii / (1 - R_ii):
//   mode 0 (occupied-space projector): pairs with exactly one of i, j below nocc get
//     (S_ij + lam_j R_ij) / (lam_j - lam_i), all others R_ij / 2;
//   mode 1 (full): pairs with |lam_j - lam_i| > delta get that quotient, the others
//     R_ij / 2 (delta: a device scalar from the caller, the cluster threshold of the
//     paper, so that no host round trip is needed).
__global__ void k_oa_correction(int n, int nocc, int mode, const double* __restrict__ delta_p,
                                const double* __restrict__ S, const double* __restrict__ R, double* __restrict__ E,
                                double* __restrict__ lam_out) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)n * n) return;
  const int i = (int)(idx / n), j = (int)(idx % n);
  const double li = __ldg(S + (long long)i * n + i) / (1.0 - __ldg(R + (long long)i * n + i));
  const double lj = __ldg(S + (long long)j * n + j) / (1.0 - __ldg(R + (long long)j * n + j));
  const double dl = lj - li;
  const double delta = delta_p ? *delta_p : 0.0;
  const double num = __ldg(S + idx) + lj * __ldg(R + idx);
  const bool sep = mode == 0 ? ((i < nocc) != (j < nocc)) : (fabs(dl) > delta);
  E[idx] = sep ? num / dl : 0.5 * __ldg(R + idx);
  if (lam_out && j == 0) lam_out[i] = li;
}

extern "C" int pcg_oa_correction(int n, int nocc, int mode, const double* delta, const double* S, const double* R,
                                 double* E, double* lam, void* stream) {
  if (n < 1 || !S || !R || !E || (mode != 0 && mode != 1)) {
    pcg_set_error("pcg_oa_correction: bad arguments");
    return PCG_ERR_ARG;
  }
  const long long total = (long long)n * n;
  k_oa_correction<<<(unsigned)((total + 255) / 256), 256, 0, (cudaStream_t)stream>>>(n, nocc, mode, delta, S, R, E,
                                                                                    lam);
  PCG_CUDA(cudaGetLastError());
  return PCG_OK;
}

// ---------------------------------------------------------------------------------
// DIIS.  state[0] = number of vectors stored so far (device int).  The new vector goes
// to slot count % cap; Bm (cap x cap) holds inner products between slots.
// ---------------------------------------------------------------------------------
__global__ void k_diis_store(long long len, int cap, const int* __restrict__ state, const double* __restrict__ F,
                             const double* __restrict__ R, double* __restrict__ focks, double* __restrict__ resids) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= len) return;
  const long long slot = state[0] % cap;
  focks[slot * len + e] = F[e];
  resids[slot * len + e] = R[e];
}

// block j: <resid slot j, R> for the slots in use after this store
__global__ void k_diis_dots(long long len, int cap, const int* __restrict__ state, const double* __restrict__ R,
                            const double* __restrict__ resids, double* __restrict__ row) {
  const int j = blockIdx.x;
  const int used = min(state[0] + 1, cap);
  if (j >= used) return;
  const double* rj = resids + (long long)j * len;
  double s = 0.0;
  for (long long e = threadIdx.x; e < len; e += blockDim.x) s = fma(__ldg(rj + e), __ldg(R + e), s);
  __shared__ double red[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) row[j] = s;
  }
}

#define DIIS_MAXCAP 32
// One thread: fold the new row into Bm, solve the C1 system over the slots in use
// (newest first; the oldest dropped while the scaled system is singular), write the
// coefficient of every slot (0 for unused) and advance the count.
__global__ void k_diis_solve(int cap, int* __restrict__ state, const double* __restrict__ row, double* __restrict__ Bm,
                             double* __restrict__ coef) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int count = state[0];
  const int slot = count % cap;
  const int used = min(count + 1, cap);
  for (int j = 0; j < used; ++j) {
    Bm[slot * cap + j] = row[j];
    Bm[j * cap + slot] = row[j];
  }
  int order[DIIS_MAXCAP];  // slots from newest to oldest
  for (int a = 0; a < used; ++a) order[a] = (slot - a + cap) % cap;
  double M[DIIS_MAXCAP + 1][DIIS_MAXCAP + 2];
  double c[DIIS_MAXCAP + 1];
  int m = used;
  bool solved = false;
  while (!solved) {
    double scale = 0.0;
    for (int a = 0; a < m; ++a) scale = fmax(scale, fabs(Bm[order[a] * cap + order[a]]));
    if (scale <= 0.0) scale = 1.0;
    for (int a = 0; a < m; ++a) {
      for (int b = 0; b < m; ++b) M[a][b] = Bm[order[a] * cap + order[b]] / scale;
      M[a][m] = -1.0;
      M[a][m + 1] = 0.0;
    }
    for (int b = 0; b < m; ++b) M[m][b] = -1.0;
    M[m][m] = 0.0;
    M[m][m + 1] = -1.0;
    bool singular = false;
    for (int col = 0; col <= m && !singular; ++col) {
      int piv = col;
      for (int r = col + 1; r <= m; ++r)
        if (fabs(M[r][col]) > fabs(M[piv][col])) piv = r;
      if (fabs(M[piv][col]) < 1e-14) { singular = true; break; }
      if (piv != col)
        for (int k = 0; k <= m + 1; ++k) { const double t = M[col][k]; M[col][k] = M[piv][k]; M[piv][k] = t; }
      for (int r = col + 1; r <= m; ++r) {
        const double f = M[r][col] / M[col][col];
        for (int k = col; k <= m + 1; ++k) M[r][k] -= f * M[col][k];
      }
    }
    if (singular) {
      if (m == 1) { c[0] = 1.0; solved = true; break; }
      --m;  // drop the oldest vector and retry
      continue;
    }
    for (int r = m; r >= 0; --r) {
      double s = M[r][m + 1];
      for (int k = r + 1; k <= m; ++k) s -= M[r][k] * c[k];
      c[r] = s / M[r][r];
    }
    solved = true;
  }
  for (int j = 0; j < cap; ++j) coef[j] = 0.0;
  for (int a = 0; a < m; ++a) coef[order[a]] = c[a];
  state[0] = count + 1;
}

__global__ void k_diis_extrapolate(long long len, int cap, const double* __restrict__ coef,
                                   const double* __restrict__ focks, double* __restrict__ Fx) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= len) return;
  double s = 0.0;
  for (int j = 0; j < cap; ++j) {
    const double cj = coef[j];
    if (cj != 0.0) s = fma(cj, focks[(long long)j * len + e], s);
  }
  Fx[e] = s;
}

extern "C" int pcg_diis_step(long long len, int cap, int* state, const double* F, const double* R, double* focks,
                             double* resids, double* Bm, double* row, double* coef, double* Fx, void* stream) {
  if (len < 1 || cap < 1 || cap > DIIS_MAXCAP || !state || !F || !R || !focks || !resids || !Bm || !row || !coef ||
      !Fx) {
    pcg_set_error("pcg_diis_step: bad arguments (1 <= cap <= 32)");
    return PCG_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const unsigned blocks = (unsigned)((len + 255) / 256);
  k_diis_store<<<blocks, 256, 0, s>>>(len, cap, state, F, R, focks, resids);
  k_diis_dots<<<cap, 1024, 0, s>>>(len, cap, state, R, resids, row);
  k_diis_solve<<<1, 32, 0, s>>>(cap, state, row, Bm, coef);
  k_diis_extrapolate<<<blocks, 256, 0, s>>>(len, cap, coef, focks, Fx);
  PCG_CUDA(cudaGetLastError());
  return PCG_OK;
}

// ------------------------------------------------------------------------------------
// Closed-shell MP2 energy sums over the transformed integrals X(i,a,j,b) = (ia|jb)
// (Methods/mp2.py:71-94), X stored b-major: X(i,a,j,b) at ((b*o + j)*v + a)*o + i, so
// that both X(i,a,j,b) and its exchange partner X(i,b,j,a) are read along i.
//   s1 = sum X(i,a,j,b)^2 / D,  s2 = sum X(i,a,j,b) X(i,b,j,a) / D,
//   D = e_i + e_j - e_a - e_b.
// Both summands are symmetric under (i,a) <-> (j,b); block p = b*o + j takes the
// pairs q = a*o + i <= p, weight 2 below the diagonal.  1/D: the FP32 reciprocal of
// the denominator formed from FP32 copies of the energies, then one Newton step
// against the FP64 denominator (relative error ~ 1e-13).  part[2p], part[2p+1]: the block's
// s1 and s2 (summed on the host side of the call, in a fixed order).
// ------------------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_mp2_pair_sums(int o, int v, const double* __restrict__ X,
                                                       const double* __restrict__ eo, const double* __restrict__ ev,
                                                       double* __restrict__ part) {
  extern __shared__ double e_sh[];                 // eo (o), then ev (v); then their FP32 copies
  float* ef = (float*)(e_sh + o + v);
  for (int t = threadIdx.x; t < o + v; t += blockDim.x) {
    const double e = t < o ? eo[t] : ev[t - o];
    e_sh[t] = e;
    ef[t] = (float)e;
  }
  __syncthreads();
  const int p = blockIdx.x, b = p / o, j = p % o;
  const double ejb = e_sh[j] - e_sh[o + b];
  const float fjb = ef[j] - ef[o + b];
  const double* Xp = X + (size_t)p * v * o;                       // X(., ., j, b)
  const int step = blockDim.x, da = step / o, di = step % o;
  int a = threadIdx.x / o, i = threadIdx.x % o;
  double s1 = 0.0, s2 = 0.0;
  // every pair q <= p with weight 1; the block total is 2 * sum - (the q = p term)
  for (int q = threadIdx.x; q <= p; q += step) {
    const double x = Xp[q];
    const double xe = X[((size_t)(a * o + j) * v + b) * o + i];   // X(i, b, j, a)
    const double d = (e_sh[i] - e_sh[o + a]) + ejb;
    // FP32 seed from the FP32 energies, one Newton step against the FP64 denominator
    double r = (double)__frcp_rn((ef[i] - ef[o + a]) + fjb);
    r = fma(r, fma(-d, r, 1.0), r);
    const double t = x * r;
    s1 = fma(x, t, s1);
    s2 = fma(xe, t, s2);
    i += di; a += da;
    if (i >= o) { i -= o; ++a; }
  }
  for (int off = 16; off; off >>= 1) {
    s1 += __shfl_xor_sync(0xffffffffu, s1, off);
    s2 += __shfl_xor_sync(0xffffffffu, s2, off);
  }
  __shared__ double red[2][8];
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) { red[0][w] = s1; red[1][w] = s2; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double r1 = 0.0, r2 = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) { r1 += red[0][k]; r2 += red[1][k]; }
    const double xd = Xp[p];                       // (jb|jb), its own exchange partner
    const double dg = xd * xd / (2.0 * ejb);
    part[2 * (size_t)p] = 2.0 * r1 - dg;
    part[2 * (size_t)p + 1] = 2.0 * r2 - dg;
  }
}

extern "C" int pcg_mp2_pair_sums(int o, int v, const double* X, const double* eo, const double* ev, double* part,
                                 void* stream) {
  if (o < 1 || v < 1 || !X || !eo || !ev || !part || (long long)o * v > 0x7fffffffLL ||
      (size_t)(o + v) * (sizeof(double) + sizeof(float)) > 200 * 1024) {
    pcg_set_error("pcg_mp2_pair_sums: bad arguments");
    return PCG_ERR_ARG;
  }
  const size_t sh = (size_t)(o + v) * (sizeof(double) + sizeof(float));
  if (sh > 48 * 1024) PCG_CUDA(cudaFuncSetAttribute(k_mp2_pair_sums, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh));
  k_mp2_pair_sums<<<o * v, 256, sh, (cudaStream_t)stream>>>(o, v, X, eo, ev, part);
  PCG_CUDA(cudaGetLastError());
  return PCG_OK;
}
