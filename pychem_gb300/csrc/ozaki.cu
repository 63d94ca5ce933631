// FP64-accurate GEMM on BF16 tensor cores by error-free operand splitting (the Ozaki
// scheme: K. Ozaki, T. Ogita, S. Oishi, S. M. Rump, "Error-free transformations of
// matrix multiplication by using fast routines of matrix multiplication and its
// applications", Numer. Algorithms 59 (2012) 95-118).
//
// C[b][m][n] (+)= sum_k A[b][m][k] B[b][k][n], all FP64.
//  1. Every row of A (over k) and column of B (over k) gets a power-of-two scale 2^e
//     with |x| < 2^e (e from the exponent field of the vector's largest |x|).  The
//     63-bit fixed-point fraction F = |x| 2^{63-e} is read off the FP64 bit pattern
//     with integer operations only and cut into s digits of beta = 7 bits (rounded at
//     the last digit), rebalanced to signed digits in [-64, 63] (the leading digit in
//     [0, 128]) and given the sign of x: x = 2^e sum_p a_p 2^{-beta p} + O(2^{e-43}).
//     |a_1| <= 128 and |a_p| <= 64 are integers that BF16 holds exactly.  No FP64
//     arithmetic is involved (GB300's FP64 pipe is ~1/60 of its FP32 pipe).
//  2. Slice products A_p B_q are integer matrices computed on the tensor cores with FP32
//     accumulation (products of 8-bit integers are exact in FP32).  Products of one level
//     L = p + q (p, q <= s, L <= s + 1) share the scale 2^{-beta L} and are summed in
//     one FP32 buffer, exact while K (2 * 2^13 + (s - 2) 2^12) < 2^24, i.e.
//     K (s + 2) < 4096 (checked; K = 298 allows s <= 11).
//  3. Every level has its own FP32 buffer; one pass combines them exactly in int64,
//     acc = sum_L P_L 2^{beta (s+1-L)} (|acc| < 2^60), and writes
//     C = acc 2^{eA + eB - beta (s+1)} (one int64->FP64 conversion per element).
// Dropped terms (p + q > s + 1) bound the relative error of an element by about
// K 2^{-beta s} of (row max of A) * (column max of B).
//
// The slice GEMMs are plain library GEMMs (cuBLAS, BF16 in, FP32 out); splitting and
// FP64 accumulation are the kernels below.
#include <cublas_v2.h>
#include <cuda_bf16.h>
#include <math.h>
#include <stdio.h>

#include "../../include/pychem_gb300.h"
#include "common.cuh"
#include "pcg_internal.h"

#define OZ_BETA 7

static cublasHandle_t g_cublas[64];

static int get_cublas(cublasHandle_t* h) {
  int dev = 0;
  PCG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) { pcg_set_error("device ordinal out of range"); return PCG_ERR_ARG; }
  if (!g_cublas[dev]) {
    if (cublasCreate(&g_cublas[dev]) != CUBLAS_STATUS_SUCCESS) { pcg_set_error("cublasCreate failed"); return PCG_ERR_CUDA; }
  }
  *h = g_cublas[dev];
  return PCG_OK;
}

// Split: one CTA per OZ_VB consecutive vectors.  Vector v = (v1, v0) holds elements
// src[v1*s1 + v0*s0 + k*ks], k < K; the CTA stages its OZ_VB x K tile in shared memory
// (coalesced along whichever of s0 / ks is 1), finds each vector's exponent, then
// writes the digits of every element to the nslice slice arrays (same layout as src).
#define OZ_VB 32
#define OZ_THREADS 256

__device__ __forceinline__ unsigned long long oz_absbits(double x) {
  return (unsigned long long)__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFull;
}

__global__ void __launch_bounds__(OZ_THREADS) k_oz_split(const double* __restrict__ src, long long n1, long long s1,
                                                         long long n0, long long s0, int K, long long ks, int nslice,
                                                         __nv_bfloat16* __restrict__ slices, long long slice_stride,
                                                         int* __restrict__ exps) {
  extern __shared__ double tile[];  // [OZ_VB][K]
  __shared__ unsigned long long vmax[OZ_VB];
  const long long nv = n1 * n0;
  const long long vbase = (long long)blockIdx.x * OZ_VB;
  const int nvl = (int)min((long long)OZ_VB, nv - vbase);
  const bool vec_fast = (s0 == 1);  // consecutive threads -> consecutive vectors
  const int total = OZ_VB * K;
  for (int idx = threadIdx.x; idx < total; idx += OZ_THREADS) {
    int vl, k;
    if (vec_fast) { vl = idx % OZ_VB; k = idx / OZ_VB; } else { vl = idx / K; k = idx % K; }
    double x = 0.0;
    if (vl < nvl) {
      const long long v = vbase + vl;
      x = src[(v / n0) * s1 + (v % n0) * s0 + (long long)k * ks];
    }
    tile[vl * K + k] = x;
  }
  __syncthreads();
  // per-vector max |x| as an integer compare of the magnitude bit patterns
  {
    const int g = OZ_THREADS / OZ_VB;  // threads per vector
    const int vl = threadIdx.x / g, lane = threadIdx.x % g;
    unsigned long long m = 0;
    for (int k = lane; k < K; k += g) m = max(m, oz_absbits(tile[vl * K + k]));
    for (int off = g / 2; off > 0; off >>= 1) m = max(m, __shfl_down_sync(0xffffffffu, m, off, g));
    if (lane == 0) vmax[vl] = m;
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < total; idx += OZ_THREADS) {
    int vl, k;
    if (vec_fast) { vl = idx % OZ_VB; k = idx / OZ_VB; } else { vl = idx / K; k = idx % K; }
    if (vl >= nvl) continue;
    const unsigned long long mb = vmax[vl];
    const int emax = (int)(mb >> 52);                 // exponent field of the vector max
    const int e = emax ? emax - 1022 : 0;             // max < 2^e
    const long long v = vbase + vl;
    if (k == 0) exps[v] = e;
    const unsigned long long u = (unsigned long long)__double_as_longlong(tile[vl * K + k]);
    const int ex = (int)((u >> 52) & 0x7FF);
    unsigned long long F = 0;
    if (ex != 0 && emax != 0) {
      const unsigned long long mant = (u & 0xFFFFFFFFFFFFFull) | (1ull << 52);
      const int sh = ex - 1012 - e;                   // F = mant 2^sh < 2^63
      if (sh >= 0) F = mant << sh;
      else if (sh > -64) F = mant >> (-sh);
    }
    int d[8];
    const int lowbit = 63 - 7 * nslice;               // first bit below the last digit
    for (int p = 1; p <= nslice; ++p) d[p - 1] = (int)((F >> (63 - 7 * p)) & 127ull);
    if (lowbit >= 1) d[nslice - 1] += (int)((F >> (lowbit - 1)) & 1ull);  // round the last digit
    int carry = 0;
    for (int p = nslice - 1; p >= 1; --p) {
      int t = d[p] + carry;
      carry = t >= 64 ? 1 : 0;
      d[p] = t - 128 * carry;
    }
    d[0] += carry;
    const bool neg = (u >> 63) != 0;
    const long long off = (v / n0) * s1 + (v % n0) * s0 + (long long)k * ks;
    for (int p = 0; p < nslice; ++p)
      slices[(long long)p * slice_stride + off] = __int2bfloat16_rn(neg ? -d[p] : d[p]);
  }
}

// C[b][m][n] (+)= (sum_L P_L[b][m][n] 2^{beta (s+1-L)}) 2^{eA[bA][m] + eB[bB][n] - beta (s+1)}
__global__ void k_oz_combine(const float* __restrict__ P, long long pstride, int nslice, double* __restrict__ C,
                             long long batch, int M, int N, long long sCb, const int* __restrict__ eA, int a_batched,
                             const int* __restrict__ eB, int b_batched, int assign) {
  const long long total = batch * (long long)M * N;
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    long long acc = 0;
    for (int L = 2; L <= nslice + 1; ++L)
      acc += __float2ll_rn(P[(long long)(L - 2) * pstride + idx]) << (OZ_BETA * (nslice + 1 - L));
    const int n = (int)(idx % N);
    const long long t = idx / N;
    const int m = (int)(t % M);
    const long long b = t / M;
    const int e = eA[(a_batched ? b * M : 0) + m] + eB[(b_batched ? b * N : 0) + n] - OZ_BETA * (nslice + 1);
    double v = 0.0;
    if (acc != 0) {
      // exact power-of-two scaling by adding to the exponent field (no FP64 multiply)
      long long bits = __double_as_longlong(__ll2double_rn(acc));
      const int ef = (int)((bits >> 52) & 0x7FF) + e;
      if (ef <= 0) v = 0.0;  // below the normal range: far under any tolerance here
      else { bits = (bits & ~(0x7FFll << 52)) | ((long long)ef << 52); v = __longlong_as_double(bits); }
    }
    double* c = C + b * sCb + (long long)m * N + n;
    *c = assign ? v : *c + v;
  }
}

static long long extent(long long nb, long long sb, long long n1, long long s1, long long n2, long long s2) {
  return (nb - 1) * sb + (n1 - 1) * s1 + (n2 - 1) * s2 + 1;
}

static size_t align256(size_t x) { return (x + 255) / 256 * 256; }

struct OzLayout {
  long long extA, extB, nvecA, nvecB, pstride;
  size_t offA, offB, offEA, offEB, offP, total;
};

static OzLayout oz_layout(const pcg_gemm_desc_t* d, int s) {
  OzLayout L;
  const long long nbA = d->sAb ? d->batch : 1, nbB = d->sBb ? d->batch : 1;
  // slice stride rounded to 128 elements so every slice starts 256-byte aligned
  L.extA = (extent(nbA, d->sAb, d->M, d->sAm, d->K, d->sAk) + 127) / 128 * 128;
  L.extB = (extent(nbB, d->sBb, d->N, d->sBn, d->K, d->sBk) + 127) / 128 * 128;
  L.nvecA = nbA * d->M;
  L.nvecB = nbB * d->N;
  size_t o = 0;
  L.offA = o; o = align256(o + (size_t)s * L.extA * 2);
  L.offB = o; o = align256(o + (size_t)s * L.extB * 2);
  L.offEA = o; o = align256(o + (size_t)L.nvecA * 4);
  L.offEB = o; o = align256(o + (size_t)L.nvecB * 4);
  L.pstride = ((long long)d->batch * d->M * d->N + 63) / 64 * 64;
  L.offP = o; o = align256(o + (size_t)s * L.pstride * 4);
  L.total = o;
  return L;
}

extern "C" size_t pcg_ozaki_workspace(const pcg_gemm_desc_t* d, int nslice) {
  if (!d || nslice < 1) return 0;
  return oz_layout(d, nslice).total;
}

extern "C" int pcg_ozaki_gemm(const pcg_gemm_desc_t* d, const double* A, const double* B, double* C, int nslice,
                              int accumulate, void* workspace, size_t ws_bytes, void* stream) {
  if (!d || !A || !B || !C || nslice < 1 || nslice > 7 || d->batch < 1 || d->M < 1 || d->N < 1 || d->K < 1) {
    pcg_set_error("pcg_ozaki_gemm: bad arguments");
    return PCG_ERR_ARG;
  }
  // exact FP32 level sums: K (2 * 2^13 + (s - 2) * 2^12) < 2^24  <=>  K (s + 2) < 4096
  if ((long long)d->K * (nslice + 2) >= 4096) {
    pcg_set_error("pcg_ozaki_gemm: K too large for exact FP32 level sums (need K * (nslice + 2) < 4096)");
    return PCG_ERR_UNSUPPORTED;
  }
  const bool a_rowk = d->sAk == 1, a_colm = d->sAm == 1;
  const bool b_rown = d->sBn == 1, b_colk = d->sBk == 1;
  if (!(a_rowk || a_colm) || !(b_rown || b_colk)) {
    pcg_set_error("pcg_ozaki_gemm: each operand needs a unit stride along one of its two matrix axes");
    return PCG_ERR_ARG;
  }
  const OzLayout L = oz_layout(d, nslice);
  if (!workspace || ws_bytes < L.total) {
    pcg_set_error("pcg_ozaki_gemm: workspace too small (query pcg_ozaki_workspace)");
    return PCG_ERR_CAPACITY;
  }
  cudaStream_t s = (cudaStream_t)stream;
  char* ws = (char*)workspace;
  __nv_bfloat16* sa = (__nv_bfloat16*)(ws + L.offA);
  __nv_bfloat16* sb = (__nv_bfloat16*)(ws + L.offB);
  int* eA = (int*)(ws + L.offEA);
  int* eB = (int*)(ws + L.offEB);
  float* P = (float*)(ws + L.offP);
  // split A: vectors (b, m) along k; B: vectors (b, n) along k
  const size_t smem = (size_t)OZ_VB * d->K * sizeof(double);
  PCG_CUDA(cudaFuncSetAttribute(k_oz_split, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  {
    const long long nb = d->sAb ? d->batch : 1;
    const long long nv = nb * d->M;
    k_oz_split<<<(unsigned)((nv + OZ_VB - 1) / OZ_VB), OZ_THREADS, smem, s>>>(A, nb, d->sAb, d->M, d->sAm, d->K,
                                                                             d->sAk, nslice, sa, L.extA, eA);
    PCG_CUDA(cudaGetLastError());
  }
  {
    const long long nb = d->sBb ? d->batch : 1;
    const long long nv = nb * d->N;
    k_oz_split<<<(unsigned)((nv + OZ_VB - 1) / OZ_VB), OZ_THREADS, smem, s>>>(B, nb, d->sBb, d->N, d->sBn, d->K,
                                                                             d->sBk, nslice, sb, L.extB, eB);
    PCG_CUDA(cudaGetLastError());
  }
  cublasHandle_t h;
  if (int rc = get_cublas(&h)) return rc;
  if (cublasSetStream(h, s) != CUBLAS_STATUS_SUCCESS) { pcg_set_error("cublasSetStream failed"); return PCG_ERR_CUDA; }
  // column-major call: C_cm (N x M, ld N) = opB(B) (N x K) * opA(A) (K x M)
  const cublasOperation_t opB = b_rown ? CUBLAS_OP_N : CUBLAS_OP_T;
  const long long ldb = b_rown ? d->sBk : d->sBn;
  const cublasOperation_t opA = a_rowk ? CUBLAS_OP_N : CUBLAS_OP_T;
  const long long lda = a_rowk ? d->sAm : d->sAk;
  const float one = 1.0f, zero = 0.0f;
  const long long total = (long long)d->batch * d->M * d->N;
  const int threads = 256;
  const int blocks = (int)((total + threads - 1) / threads > 152 * 64 ? 152 * 64 : (total + threads - 1) / threads);
  for (int lev = 2; lev <= nslice + 1; ++lev) {
    bool first = true;
    float* PL = P + (size_t)(lev - 2) * L.pstride;
    for (int p = 1; p <= nslice; ++p) {
      const int q = lev - p;
      if (q < 1 || q > nslice) continue;
      const cublasStatus_t st = cublasGemmStridedBatchedEx(
          h, opB, opA, d->N, d->M, d->K, &one, sb + (size_t)(q - 1) * L.extB, CUDA_R_16BF, (int)ldb, d->sBb,
          sa + (size_t)(p - 1) * L.extA, CUDA_R_16BF, (int)lda, d->sAb, first ? &zero : &one, PL, CUDA_R_32F, d->N,
          (long long)d->M * d->N, d->batch, CUBLAS_COMPUTE_32F, CUBLAS_GEMM_DEFAULT);
      if (st != CUBLAS_STATUS_SUCCESS) {
        char msg[96];
        snprintf(msg, sizeof(msg), "cublasGemmStridedBatchedEx failed (%d)", (int)st);
        pcg_set_error(msg);
        return PCG_ERR_CUDA;
      }
      first = false;
    }
  }
  k_oz_combine<<<blocks, threads, 0, s>>>(P, L.pstride, nslice, C, d->batch, d->M, d->N, d->sCb, eA, d->sAb ? 1 : 0,
                                          eB, d->sBb ? 1 : 0, accumulate ? 0 : 1);
  PCG_CUDA(cudaGetLastError());
  return PCG_OK;
}
