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
//     L = p + q (p, q <= s, L <= s + 1) share the scale 2^{-beta L}; the slices are
//     stored so that a level is ONE GEMM over the concatenated inner dimension
//     (A_{p_lo} .. A_{p_hi}) x (B_{L-p_lo}; ..; B_{L-p_hi}): A slices row-interleaved
//     [vector][p][k], B slices in descending order [batch][s - q][k][n].  The level sum
//     is exact in FP32 while K (2 * 2^13 + (s - 2) 2^12) < 2^24, i.e. K (s + 2) < 4096
//     (checked; K = 298 allows s <= 11).
//  3. Every level has its own FP32 buffer; one pass combines them exactly in int64,
//     acc = sum_L P_L 2^{beta (s+1-L)} (|acc| < 2^60), and writes
//     C = acc 2^{eA + eB - beta (s+1)} (acc rounded to FP64 with integer operations).
// Dropped terms (p + q > s + 1) bound the relative error of an element by about
// K 2^{-beta s} of (row max of A) * (column max of B).
//
// The level GEMMs are plain library GEMMs (cuBLAS, BF16 in, FP32 out); splitting and
// FP64 accumulation are the kernels below.
#include <cublas_v2.h>
#include <cuda_bf16.h>
#include <math.h>
#include <stdio.h>

#include "../../include/pychem_gb300.h"
#include "common.cuh"
#include "pcg_internal.h"
#include "ozaki_common.cuh"

#define OZ_BETA 7
#define OZ_THREADS 256

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

// Split.  A vector is one row of A or one column of B over k: vector (v1, v0) holds
// src[v1*s1 + v0*s0 + k*ks], k < K (v1 the batch).  Its exponent e (max |x| < 2^e)
// comes from an integer max of the magnitude bit patterns; the digits of each element
// then go to the slice layout of the operand's role:
//   role A: out[((v1 * n0 + v0) * NS + p - 1) * K + k]
//   role B: out[((v1 * NS + NS - p) * K + k) * n0 + v0]
template <int NS>
__device__ __forceinline__ long long oz_out(bool roleA, long long v1, long long v0, long long n0, int K, int p, int k) {
  return roleA ? ((v1 * n0 + v0) * NS + p - 1) * K + k : ((v1 * NS + NS - p) * (long long)K + k) * n0 + v0;
}

// Vectors contiguous (s0 == 1): one thread per vector; each k is one coalesced row of
// consecutive vectors.  Two streaming passes: k_oz_vmax_v writes every vector's
// exponent, then k_oz_split_v writes the digits.
__global__ void __launch_bounds__(OZ_THREADS) k_oz_vmax_v(const double* __restrict__ src, long long n1,
                                                          long long s1, long long n0, int K, long long ks,
                                                          int* __restrict__ exps) {
  const long long chunks = (n0 + OZ_THREADS - 1) / OZ_THREADS;
  const long long v1 = blockIdx.x / chunks;
  const long long v0 = (blockIdx.x % chunks) * OZ_THREADS + threadIdx.x;
  if (v1 >= n1 || v0 >= n0) return;
  const double* x = src + v1 * s1 + v0;
  unsigned long long m = 0;
#pragma unroll 16
  for (int k = 0; k < K; ++k) m = max(m, oz_absbits(__ldg(x + (long long)k * ks)));
  exps[v1 * n0 + v0] = (int)(m >> 52);   // exponent field of the max (converted below)
}

template <int NS>
__global__ void __launch_bounds__(OZ_THREADS) k_oz_split_v(const double* __restrict__ src, long long n1,
                                                           long long s1, long long n0, int K, long long ks,
                                                           int roleA, __nv_bfloat16* __restrict__ out,
                                                           int* __restrict__ exps) {
  const long long chunks = (n0 + OZ_THREADS - 1) / OZ_THREADS;
  const long long v1 = blockIdx.x / chunks;
  const long long v0 = (blockIdx.x % chunks) * OZ_THREADS + threadIdx.x;
  if (v1 >= n1 || v0 >= n0) return;
  const double* x = src + v1 * s1 + v0;
  const int emax = exps[v1 * n0 + v0];
  exps[v1 * n0 + v0] = emax ? emax - 1022 : 0;
#pragma unroll 4
  for (int k = 0; k < K; ++k) {
    int d[NS];
    oz_digits<NS>(__ldg(x + (long long)k * ks), emax, d);
#pragma unroll
    for (int p = 1; p <= NS; ++p) out[oz_out<NS>(roleA, v1, v0, n0, K, p, k)] = __int2bfloat16_rn(d[p - 1]);
  }
}

// The same two passes with 4 consecutive vectors per thread (32-byte loads, 8-byte
// digit stores): used for role B when n0, s1 and ks are multiples of 4 and src is
// 32-byte aligned, so a CTA reads 8 KB of one row per k.
__global__ void __launch_bounds__(OZ_THREADS) k_oz_vmax_v4(const double* __restrict__ src, long long n1,
                                                           long long s1, long long n0, int K, long long ks,
                                                           int* __restrict__ exps) {
  const long long chunks = (n0 + 4 * OZ_THREADS - 1) / (4 * OZ_THREADS);
  const long long v1 = blockIdx.x / chunks;
  const long long v0 = ((blockIdx.x % chunks) * OZ_THREADS + threadIdx.x) * 4;
  if (v1 >= n1 || v0 >= n0) return;
  const double* x = src + v1 * s1 + v0;
  unsigned long long m0 = 0, m1 = 0, m2 = 0, m3 = 0;
#pragma unroll 8
  for (int k = 0; k < K; ++k) {
    const double2 qa = __ldg((const double2*)(x + (long long)k * ks));
    const double2 qb = __ldg((const double2*)(x + (long long)k * ks) + 1);
    m0 = max(m0, oz_absbits(qa.x)); m1 = max(m1, oz_absbits(qa.y));
    m2 = max(m2, oz_absbits(qb.x)); m3 = max(m3, oz_absbits(qb.y));
  }
  *(int4*)(exps + v1 * n0 + v0) = make_int4((int)(m0 >> 52), (int)(m1 >> 52), (int)(m2 >> 52), (int)(m3 >> 52));
}

template <int NS>
__global__ void __launch_bounds__(OZ_THREADS) k_oz_split_v4(const double* __restrict__ src, long long n1,
                                                            long long s1, long long n0, int K, long long ks,
                                                            __nv_bfloat16* __restrict__ out, int* __restrict__ exps) {
  const long long chunks = (n0 + 4 * OZ_THREADS - 1) / (4 * OZ_THREADS);
  const long long v1 = blockIdx.x / chunks;
  const long long v0 = ((blockIdx.x % chunks) * OZ_THREADS + threadIdx.x) * 4;
  if (v1 >= n1 || v0 >= n0) return;
  const double* x = src + v1 * s1 + v0;
  int4 em = *(const int4*)(exps + v1 * n0 + v0);
  *(int4*)(exps + v1 * n0 + v0) = make_int4(em.x ? em.x - 1022 : 0, em.y ? em.y - 1022 : 0, em.z ? em.z - 1022 : 0,
                                            em.w ? em.w - 1022 : 0);
#pragma unroll 2
  for (int k = 0; k < K; ++k) {
    const double2 qa = __ldg((const double2*)(x + (long long)k * ks));
    const double2 qb = __ldg((const double2*)(x + (long long)k * ks) + 1);
    int d0[NS], d1[NS], d2[NS], d3[NS];
    oz_digits<NS>(qa.x, em.x, d0);
    oz_digits<NS>(qa.y, em.y, d1);
    oz_digits<NS>(qb.x, em.z, d2);
    oz_digits<NS>(qb.y, em.w, d3);
#pragma unroll
    for (int p = 1; p <= NS; ++p) {
      __nv_bfloat162 lo = __halves2bfloat162(__int2bfloat16_rn(d0[p - 1]), __int2bfloat16_rn(d1[p - 1]));
      __nv_bfloat162 hi = __halves2bfloat162(__int2bfloat16_rn(d2[p - 1]), __int2bfloat16_rn(d3[p - 1]));
      uint2 w;
      w.x = *(unsigned*)&lo;
      w.y = *(unsigned*)&hi;
      *(uint2*)(out + ((v1 * NS + NS - p) * (long long)K + k) * n0 + v0) = w;
    }
  }
}

// k contiguous (ks == 1): one warp per vector, lanes over k.
template <int NS>
__global__ void __launch_bounds__(OZ_THREADS) k_oz_split_k(const double* __restrict__ src, long long n1,
                                                           long long s1, long long n0, long long s0, int K,
                                                           int roleA, __nv_bfloat16* __restrict__ out,
                                                           int* __restrict__ exps) {
  const long long v = (long long)blockIdx.x * (OZ_THREADS / 32) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (v >= n1 * n0) return;
  const long long v1 = v / n0, v0 = v % n0;
  const double* x = src + v1 * s1 + v0 * s0;
  unsigned long long m = 0;
  for (int k = lane; k < K; k += 32) m = max(m, oz_absbits(__ldg(x + k)));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  const int emax = (int)(m >> 52);
  if (lane == 0) exps[v] = emax ? emax - 1022 : 0;
  for (int k = lane; k < K; k += 32) {
    int d[NS];
    oz_digits<NS>(__ldg(x + k), emax, d);
#pragma unroll
    for (int p = 1; p <= NS; ++p) out[oz_out<NS>(roleA, v1, v0, n0, K, p, k)] = __int2bfloat16_rn(d[p - 1]);
  }
}

// C[b][m][n] (+)= (sum_L P_L[b][m][n] 2^{beta (s+1-L)}) 2^{eA[bA][m] + eB[bB][n] - beta (s+1)}
// One CTA per row r = b * M + m and chunk of 4 * OZ_THREADS columns.
#define OZ_COMBINE_COLS (4 * OZ_THREADS)
__global__ void __launch_bounds__(OZ_THREADS) k_oz_combine(const float* __restrict__ P, long long pstride, int nslice,
                                                           double* __restrict__ C, long long rows, int M, int N,
                                                           long long sCb, const int* __restrict__ eA, int a_batched,
                                                           const int* __restrict__ eB, int b_batched, int assign) {
  const long long nch = (N + OZ_COMBINE_COLS - 1) / OZ_COMBINE_COLS;
  const long long r = blockIdx.x / nch;
  if (r >= rows) return;
  const int c0 = (int)(blockIdx.x % nch) * OZ_COMBINE_COLS;
  const long long b = r / M;
  const int m = (int)(r % M);
  const int ea = eA[(a_batched ? b * M : 0) + m] - OZ_BETA * (nslice + 1);
  const int* eb = eB + (b_batched ? b * N : 0);
  const float* Pr = P + r * N;
  double* Cr = C + b * sCb + (long long)m * N;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int n = c0 + j * OZ_THREADS + threadIdx.x;
    if (n >= N) break;
    // level sums are integers below 2^24: FP32 -> int32 conversions, int64 shifts
    long long acc = 0;
    for (int L = 2; L <= nslice + 1; ++L)
      acc += (long long)__float2int_rn(__ldg(Pr + (long long)(L - 2) * pstride + n)) << (OZ_BETA * (nslice + 1 - L));
    const int e = ea + __ldg(eb + n);
    const double v = oz_ll_scaled(acc, e);
    Cr[n] = assign ? v : Cr[n] + v;
  }
}

// The same with 4 consecutive columns per thread (16-byte level loads and stores)
// when N and sCb are multiples of 4.
__global__ void __launch_bounds__(OZ_THREADS) k_oz_combine4(const float* __restrict__ P, long long pstride,
                                                            int nslice, double* __restrict__ C, long long rows, int M,
                                                            int N, long long sCb, const int* __restrict__ eA,
                                                            int a_batched, const int* __restrict__ eB, int b_batched,
                                                            int assign) {
  const long long nch = (N + OZ_COMBINE_COLS - 1) / OZ_COMBINE_COLS;
  const long long r = blockIdx.x / nch;
  if (r >= rows) return;
  const int n = (int)(blockIdx.x % nch) * OZ_COMBINE_COLS + 4 * threadIdx.x;
  if (n >= N) return;
  const long long b = r / M;
  const int m = (int)(r % M);
  const int ea = eA[(a_batched ? b * M : 0) + m] - OZ_BETA * (nslice + 1);
  const int4 eb = __ldg((const int4*)(eB + (b_batched ? b * N : 0) + n));
  const float* Pr = P + r * N + n;
  long long a0 = 0, a1 = 0, a2 = 0, a3 = 0;
  for (int L = 2; L <= nslice + 1; ++L) {
    const float4 q = __ldg((const float4*)(Pr + (long long)(L - 2) * pstride));
    const int sh = OZ_BETA * (nslice + 1 - L);
    a0 += (long long)__float2int_rn(q.x) << sh;
    a1 += (long long)__float2int_rn(q.y) << sh;
    a2 += (long long)__float2int_rn(q.z) << sh;
    a3 += (long long)__float2int_rn(q.w) << sh;
  }
  double2 v0 = make_double2(oz_ll_scaled(a0, ea + eb.x), oz_ll_scaled(a1, ea + eb.y));
  double2 v1 = make_double2(oz_ll_scaled(a2, ea + eb.z), oz_ll_scaled(a3, ea + eb.w));
  double2* c = (double2*)(C + b * sCb + (long long)m * N + n);
  if (!assign) {
    const double2 o0 = c[0], o1 = c[1];
    v0.x += o0.x; v0.y += o0.y; v1.x += o1.x; v1.y += o1.y;
  }
  c[0] = v0;
  c[1] = v1;
}

static size_t align256(size_t x) { return (x + 255) / 256 * 256; }

struct OzLayout {
  long long extA, extB, nvecA, nvecB, pstride;
  size_t offA, offB, offEA, offEB, offP, total;
};

static OzLayout oz_layout(const pcg_gemm_desc_t* d, int s) {
  OzLayout L;
  const long long nbA = d->sAb ? d->batch : 1, nbB = d->sBb ? d->batch : 1;
  L.nvecA = nbA * d->M;
  L.nvecB = nbB * d->N;
  // compact slice arrays: s digits of every element of every vector
  L.extA = (L.nvecA * (long long)d->K + 127) / 128 * 128;
  L.extB = (L.nvecB * (long long)d->K + 127) / 128 * 128;
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

template <int NS>
static void oz_launch_split(const double* src, long long nb, long long sb, long long nv0, long long sv0, long long sk,
                            int K, int roleA, __nv_bfloat16* out, int* ex, cudaStream_t s) {
  // by k when k is contiguous and the vectors are not (or for A, whose slices run along k)
  if (sk == 1 && (roleA || sv0 != 1)) {
    const long long per = OZ_THREADS / 32;
    k_oz_split_k<NS><<<(unsigned)((nb * nv0 + per - 1) / per), OZ_THREADS, 0, s>>>(src, nb, sb, nv0, sv0, K, roleA,
                                                                                  out, ex);
  } else if (!roleA && nv0 % 4 == 0 && (nb == 1 || sb % 4 == 0) && sk % 4 == 0 && ((size_t)src & 31) == 0) {
    const long long chunks = (nv0 + 4 * OZ_THREADS - 1) / (4 * OZ_THREADS);
    k_oz_vmax_v4<<<(unsigned)(nb * chunks), OZ_THREADS, 0, s>>>(src, nb, sb, nv0, K, sk, ex);
    k_oz_split_v4<NS><<<(unsigned)(nb * chunks), OZ_THREADS, 0, s>>>(src, nb, sb, nv0, K, sk, out, ex);
  } else {
    const long long chunks = (nv0 + OZ_THREADS - 1) / OZ_THREADS;
    k_oz_vmax_v<<<(unsigned)(nb * chunks), OZ_THREADS, 0, s>>>(src, nb, sb, nv0, K, sk, ex);
    k_oz_split_v<NS><<<(unsigned)(nb * chunks), OZ_THREADS, 0, s>>>(src, nb, sb, nv0, K, sk, roleA, out, ex);
  }
}

static int oz_split(int nslice, const double* src, long long nb, long long sb, long long nv0, long long sv0,
                    long long sk, int K, int roleA, __nv_bfloat16* out, int* ex, cudaStream_t s) {
  switch (nslice) {
    case 1: oz_launch_split<1>(src, nb, sb, nv0, sv0, sk, K, roleA, out, ex, s); break;
    case 2: oz_launch_split<2>(src, nb, sb, nv0, sv0, sk, K, roleA, out, ex, s); break;
    case 3: oz_launch_split<3>(src, nb, sb, nv0, sv0, sk, K, roleA, out, ex, s); break;
    case 4: oz_launch_split<4>(src, nb, sb, nv0, sv0, sk, K, roleA, out, ex, s); break;
    case 5: oz_launch_split<5>(src, nb, sb, nv0, sv0, sk, K, roleA, out, ex, s); break;
    case 6: oz_launch_split<6>(src, nb, sb, nv0, sv0, sk, K, roleA, out, ex, s); break;
    case 7: oz_launch_split<7>(src, nb, sb, nv0, sv0, sk, K, roleA, out, ex, s); break;
    default: pcg_set_error("pcg_ozaki_gemm: nslice out of range"); return PCG_ERR_ARG;
  }
  PCG_CUDA(cudaGetLastError());
  return PCG_OK;
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
  if (!(d->sAk == 1 || d->sAm == 1) || !(d->sBn == 1 || d->sBk == 1)) {
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
  const long long nbA = d->sAb ? d->batch : 1, nbB = d->sBb ? d->batch : 1;
  if (int rc = oz_split(nslice, A, nbA, d->sAb, d->M, d->sAm, d->sAk, d->K, 1, sa, eA, s)) return rc;
  if (int rc = oz_split(nslice, B, nbB, d->sBb, d->N, d->sBn, d->sBk, d->K, 0, sb, eB, s)) return rc;
  cublasHandle_t h;
  if (int rc = get_cublas(&h)) return rc;
  if (cublasSetStream(h, s) != CUBLAS_STATUS_SUCCESS) { pcg_set_error("cublasSetStream failed"); return PCG_ERR_CUDA; }
  // level L = one GEMM over the inner dimension K_L = (p_hi - p_lo + 1) K; column-major
  // call: P_L (N x M, ld N) = Bcat (N x K_L, ld N) * Acat (K_L x M, ld s K)
  const float one = 1.0f, zero = 0.0f;
  const long long K = d->K;
  for (int lev = 2; lev <= nslice + 1; ++lev) {
    const int p_lo = lev - nslice > 1 ? lev - nslice : 1;
    const int p_hi = lev - 1 < nslice ? lev - 1 : nslice;
    const int kl = (p_hi - p_lo + 1) * (int)K;
    const __nv_bfloat16* Bcat = sb + (size_t)(nslice - lev + p_lo) * K * d->N;
    const __nv_bfloat16* Acat = sa + (size_t)(p_lo - 1) * K;
    float* PL = P + (size_t)(lev - 2) * L.pstride;
    const cublasStatus_t st = cublasGemmStridedBatchedEx(
        h, CUBLAS_OP_N, CUBLAS_OP_N, d->N, d->M, kl, &one, Bcat, CUDA_R_16BF, d->N,
        d->sBb ? (long long)nslice * K * d->N : 0, Acat, CUDA_R_16BF, (int)(nslice * K),
        d->sAb ? (long long)d->M * nslice * K : 0, &zero, PL, CUDA_R_32F, d->N, (long long)d->M * d->N, d->batch,
        CUBLAS_COMPUTE_32F, CUBLAS_GEMM_DEFAULT);
    if (st != CUBLAS_STATUS_SUCCESS) {
      char msg[96];
      snprintf(msg, sizeof(msg), "cublasGemmStridedBatchedEx failed (%d)", (int)st);
      pcg_set_error(msg);
      return PCG_ERR_CUDA;
    }
  }
  const long long rows = (long long)d->batch * d->M;
  const long long nch = (d->N + OZ_COMBINE_COLS - 1) / OZ_COMBINE_COLS;
  if (d->N % 4 == 0 && d->sCb % 4 == 0 && ((size_t)C & 31) == 0)
    k_oz_combine4<<<(unsigned)(rows * nch), OZ_THREADS, 0, s>>>(P, L.pstride, nslice, C, rows, d->M, d->N, d->sCb, eA,
                                                                 d->sAb ? 1 : 0, eB, d->sBb ? 1 : 0, accumulate ? 0 : 1);
  else
    k_oz_combine<<<(unsigned)(rows * nch), OZ_THREADS, 0, s>>>(P, L.pstride, nslice, C, rows, d->M, d->N, d->sCb, eA,
                                                                d->sAb ? 1 : 0, eB, d->sBb ? 1 : 0, accumulate ? 0 : 1);
  PCG_CUDA(cudaGetLastError());
  return PCG_OK;
}
