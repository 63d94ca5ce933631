// FP64-accurate GEMM on the tcgen05 tensor cores, every Ozaki level in one kernel.
//
//   C[m*sCm + n*sCn] (+)= sum_k X[m*ldx + k] * Y[k*sYk + n*sYn]      (all FP64)
//
// The scheme is the one of ozaki.cu (K. Ozaki, T. Ogita, S. Oishi, S. M. Rump, Numer.
// Algorithms 59 (2012) 95-118): each row of X and column of Y gets a power-of-two
// scale and NS signed 7-bit digits (exact in BF16); products of digit slices are exact
// integers in FP32; the level sums P_L = sum_{p+q=L} X_p Y_q are combined exactly in
// int64.  What this kernel changes is where the work happens:
//
//  * X, the large operand (millions of rows in the MP2 transforms), is read once as
//    FP64 from global memory and split on the fly: sixteen producer warps load a 128-row
//    by 32-column chunk, cut it into NS digit slices and store them BF16, K-major and
//    64-byte swizzled, straight into the shared-memory operand tiles (no BF16 copy of
//    X in global memory).  The exponent of each row comes from a first pass over the
//    CTA's rows (the re-read is served by L2).
//  * Y, the small operand (C_occ or C_vir: a few hundred columns), is split once by
//    k_ozt_split_y into K-major BF16 slices in the caller's workspace (slice-major,
//    [p][n][k]) and brought into shared memory tile by tile by the tensor memory
//    accelerator (cp.async.bulk.tensor, 64-byte swizzle, completion counted on the
//    stage's mbarrier).
//  * One thread issues tcgen05.mma (M = 128, N = BN, K = 16, BF16 in, FP32 out) for
//    every slice pair with p + q <= NS + 1 into NS accumulators in tensor memory, one
//    per level (NS * BN <= 512 columns), over a two-stage mbarrier pipeline.
//  * The producer warps then read the level accumulators (tcgen05.ld), combine them in
//    int64, scale by 2^{eX + eY} and write FP64 C with any strides (sCm = 1 gives
//    coalesced stores of the transposed product, which is how the MP2 transforms chain).
//
// Level sums are exact while K (NS + 2) < 4096.  Every mbarrier wait is bounded; a CTA
// that gives up sets the error flag in the workspace, drains its MMAs, frees its
// tensor memory and returns.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <stdio.h>

#include "../../include/pychem_gb300.h"
#include "common.cuh"
#include "ozaki_common.cuh"
#include "pcg_internal.h"
#include "umma.cuh"

#define OZT_BM 128
#define OZT_BK 32
#define OZT_PROD_WARPS 16
#define OZT_PROD (OZT_PROD_WARPS * 32)
#define OZT_THREADS (OZT_PROD + 32)
#define OZT_WAIT (1u << 24)

template <int NS, int BN>
struct OztCfg {
  static constexpr int XT = OZT_BM * OZT_BK * 2;  // one X slice tile (bytes)
  static constexpr int YT = BN * OZT_BK * 2;      // one Y slice tile
  static constexpr int STAGE = NS * (XT + YT);
  static constexpr int SMEM = 2 * STAGE + 1024 + 1024;  // two stages, alignment slack, barriers and exponents
  static_assert(NS * BN <= 512, "level accumulators exceed tensor memory");
  static_assert(BN % 16 == 0 && BN >= 16 && BN <= 256, "MMA N");
  static_assert(YT % 512 == 0, "Y tiles must stay 512-byte aligned");
};

struct OztWs {  // workspace header (device): error flag, then exponents of Y and its slices
  int err;
};

// Y slices: ys[(p * Npad + n) * Kp + k] (BF16, zero for k >= K and n >= N), ey[n]: one
// warp per column n, lanes over k.
template <int NS>
__global__ void k_ozt_split_y(const double* __restrict__ Y, long long sYk, long long sYn, int K, int N, int Npad,
                              int Kp, __nv_bfloat16* __restrict__ ys, int* __restrict__ ey) {
  const int n = blockIdx.x * 8 + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (n >= Npad) return;
  __nv_bfloat16* out = ys + (size_t)n * Kp;
  const size_t pstride = (size_t)Npad * Kp;
  if (n >= N) {
    for (int i = lane; i < NS * Kp; i += 32) out[(i / Kp) * pstride + i % Kp] = __float2bfloat16(0.0f);
    if (lane == 0) ey[n] = 0;
    return;
  }
  unsigned long long mx = 0;
  for (int k = lane; k < K; k += 32) mx = max(mx, oz_absbits(__ldg(Y + k * sYk + n * sYn)));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  const int emax = (int)(mx >> 52);
  if (lane == 0) ey[n] = emax ? emax - 1022 : 0;
  for (int k = lane; k < Kp; k += 32) {
    int d[NS];
    if (k < K) {
      oz_digits<NS>(__ldg(Y + k * sYk + n * sYn), emax, d);
    } else {
#pragma unroll
      for (int p = 0; p < NS; ++p) d[p] = 0;
    }
#pragma unroll
    for (int p = 0; p < NS; ++p) out[p * pstride + k] = __int2bfloat16_rn(d[p]);
  }
}

// the 8 consecutive FP64 values of row m from column kb (zero outside [0, K) or m >= M)
__device__ __forceinline__ void ozt_load8(const double* __restrict__ X, long long ldx, long long m, long long M, int kb,
                                          int K, bool vec, double (&v)[8]) {
  if (m < M && vec && kb + 8 <= K) {
    const double2* src = (const double2*)(X + m * ldx + kb);
#pragma unroll
    for (int h = 0; h < 4; ++h) {
      const double2 q = __ldg(src + h);
      v[2 * h] = q.x;
      v[2 * h + 1] = q.y;
    }
  } else if (m < M) {
    const double* src = X + m * ldx + kb;
#pragma unroll
    for (int j = 0; j < 8; ++j) v[j] = (kb + j < K) ? __ldg(src + j) : 0.0;
  } else {
#pragma unroll
    for (int j = 0; j < 8; ++j) v[j] = 0.0;
  }
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int c0, int c1, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          dst),
      "l"((uint64_t)map), "r"(c0), "r"(c1), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

template <int NS, int BN>
__global__ void __launch_bounds__(OZT_THREADS, 1)
    k_ozt_gemm(long long M, int N, int K, int Kp, int Npad, const double* __restrict__ X, long long ldx,
               const __grid_constant__ CUtensorMap ymap, const int* __restrict__ ey, double* __restrict__ C,
               long long sCm, long long sCn, int accumulate, int* __restrict__ err) {
  using Cfg = OztCfg<NS, BN>;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* sm = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint8_t* tiles = sm;                                        // [stage][X slices | Y slices]
  uint64_t* bars = (uint64_t*)(sm + 2 * Cfg::STAGE);  // full[2], empty[2], done, drain, ycopy[2]
  uint32_t* tmem_slot = (uint32_t*)(bars + 8);
  volatile int* abort_s = (volatile int*)(tmem_slot + 1);
  int* ex_s = (int*)(tmem_slot + 4);                           // 128 row exponent fields

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // linear grid, the N tiles of one row tile adjacent (they share its X rows in L2)
  const int ntn = (N + BN - 1) / BN;
  const long long m0 = (long long)(blockIdx.x / ntn) * OZT_BM;
  const int n0 = (int)(blockIdx.x % ntn) * BN;
  const int nchunk = Kp / OZT_BK;

  if (threadIdx.x == 0) {
    // full: every producer thread; ycopy: the expect_tx arrival of the thread that issues
    // the Y copies, completed by their bytes
    for (int i = 0; i < 2; ++i) {
      mbar_init(&bars[i], OZT_PROD);
      mbar_init(&bars[2 + i], 1);
      mbar_init(&bars[6 + i], 1);
    }
    mbar_init(&bars[4], 1);
    mbar_init(&bars[5], 1);
    *abort_s = 0;
    mbar_fence_init();
  }
  if (warp == OZT_PROD_WARPS) tmem_alloc(tmem_slot, 512);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp < OZT_PROD_WARPS) {
    const int t = threadIdx.x;
    const bool vec = (ldx % 2 == 0) && (((uintptr_t)X & 15) == 0);
    // ---- exponents of the CTA's 128 rows of X: four threads per row, each over a
    // quarter of the row (even boundaries, so 16-byte loads stay aligned)
    {
      const int r = t >> 2, h = t & 3;
      const long long m = m0 + r;
      const int kq = ((K + 3) / 4 + 1) & ~1;
      const int klo = h * kq < K ? h * kq : K, khi = (h + 1) * kq < K ? (h + 1) * kq : K;
      unsigned long long mx = 0;
      if (m < M && klo < khi) {
        const double* row = X + m * ldx;
        int k = klo;
        if (vec) {
#pragma unroll 8
          for (; k + 2 <= khi; k += 2) {
            const double2 q = __ldg((const double2*)(row + k));
            mx = max(mx, max(oz_absbits(q.x), oz_absbits(q.y)));
          }
        }
        for (; k < khi; ++k) mx = max(mx, oz_absbits(__ldg(row + k)));
      }
      mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, 1));
      mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, 2));
      if (h == 0) ex_s[r] = (int)(mx >> 52);
    }
    asm volatile("bar.sync 1, %0;" ::"r"(OZT_PROD));
    // this thread's 8-column item of every chunk: row r, column group g
    const int g = t & 3, r = t >> 2;
    const int emax = ex_s[r];
    const uint32_t off = sw64_offset(r, g);
    bool ok = true;
    int ycopies[2] = {0, 0};  // Y copies issued per stage (thread 0)
    for (int c = 0; c < nchunk; ++c) {
      const int st = c & 1;
      const int k0 = c * OZT_BK;
      double v[8];
      ozt_load8(X, ldx, m0 + r, M, k0 + 8 * g, K, vec, v);   // issued before the wait
      if (c >= 2 && !mbar_wait(&bars[2 + st], ((c >> 1) + 1) & 1, OZT_WAIT, abort_s)) { ok = false; break; }
      uint8_t* xt = tiles + st * Cfg::STAGE;
      uint8_t* yt = xt + NS * Cfg::XT;
      if (t == 0) {  // Y slices of this chunk by TMA
        ++ycopies[st];
        mbar_arrive_expect_tx(&bars[6 + st], NS * Cfg::YT);
#pragma unroll 1
        for (int p = 0; p < NS; ++p) tma_load_2d(smem_u32(yt + p * Cfg::YT), &ymap, k0, p * Npad + n0, &bars[6 + st]);
      }
      unsigned w[4][NS];
#pragma unroll
      for (int hh = 0; hh < 4; ++hh) oz_digits_bf16x2<NS>(v[2 * hh], v[2 * hh + 1], emax, w[hh]);
#pragma unroll
      for (int p = 0; p < NS; ++p)
        *(uint4*)(xt + p * Cfg::XT + off) = make_uint4(w[0][p], w[1][p], w[2][p], w[3][p]);
      fence_proxy_async_smem();
      mbar_arrive(&bars[st]);
    }
    if (!ok) { *abort_s = 1; atomicExch(err, 1); }
    if (t == 0 && *abort_s) {  // let this thread's Y copies land before the CTA exits
      volatile int keep_waiting = 0;
      for (int i = 0; i < 2; ++i)
        if (ycopies[i]) mbar_wait(&bars[6 + i], (ycopies[i] - 1) & 1, OZT_WAIT, &keep_waiting);
    }
    // ---- epilogue: wait for the last MMAs, combine the levels, write C
    if (ok && mbar_wait(&bars[4], 0, OZT_WAIT, abort_s)) {
      tc_fence_after();
      const int lg = warp & 3, quarter = warp >> 2;
      const int re = 32 * lg + lane;
      const long long m = m0 + re;
      const int eme = ex_s[re];
      const int ex = (eme ? eme - 1022 : 0) - OZ_BETA * (NS + 1);
      const uint32_t trow = tmem + ((uint32_t)(32 * lg) << 16);
#pragma unroll 1
      for (int cb = 8 * quarter; cb < BN; cb += 32) {
        float P[NS][8];
#pragma unroll
        for (int L = 0; L < NS; ++L) tmem_ld8(trow + L * BN + cb, P[L]);
        tmem_wait_ld();
        if (m < M) {
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const int n = n0 + cb + j;
            if (n >= N) break;
            long long acc = 0;
#pragma unroll
            for (int L = 0; L < NS; ++L) acc += (long long)__float2int_rn(P[L][j]) << (OZ_BETA * (NS - 1 - L));
            const double val = oz_ll_scaled(acc, ex + __ldg(ey + n));
            double* cp = C + m * sCm + (long long)n * sCn;
            *cp = accumulate ? *cp + val : val;
          }
        }
      }
    } else {
      *abort_s = 1;
      atomicExch(err, 1);
    }
  } else if (lane == 0) {
    // ---- MMA issuer
    const uint32_t idesc = idesc_bf16_f32(OZT_BM, BN);
    unsigned inited = 0;
    bool ok = true;
    for (int c = 0; c < nchunk; ++c) {
      const int st = c & 1;
      if (!mbar_wait(&bars[st], (c >> 1) & 1, OZT_WAIT, abort_s) ||
          !mbar_wait(&bars[6 + st], (c >> 1) & 1, OZT_WAIT, abort_s)) {
        ok = false;
        break;
      }
      tc_fence_after();
      const uint32_t xa = smem_u32(tiles + st * Cfg::STAGE);
      const uint32_t ya = xa + NS * Cfg::XT;
#pragma unroll
      for (int kk = 0; kk < OZT_BK / 16; ++kk) {
#pragma unroll
        for (int p = 0; p < NS; ++p)
#pragma unroll
          for (int q = 0; q < NS - p; ++q) {
            const int L = p + q;
            const uint64_t ad = sdesc_k_sw64(xa + p * Cfg::XT + kk * 32);
            const uint64_t bd = sdesc_k_sw64(ya + q * Cfg::YT + kk * 32);
            umma_bf16(tmem + L * BN, ad, bd, idesc, (inited >> L) & 1u);
            inited |= 1u << L;
          }
      }
      umma_commit(&bars[2 + st]);
    }
    if (ok) {
      umma_commit(&bars[4]);
    } else {
      *abort_s = 1;
      atomicExch(err, 2);
      umma_commit(&bars[5]);  // drain what was issued before freeing tensor memory
      volatile int keep_waiting = 0;
      mbar_wait(&bars[5], 0, OZT_WAIT, &keep_waiting);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == OZT_PROD_WARPS) {
    __syncwarp();
    tc_fence_after();
    tmem_dealloc(tmem, 512);
  }
}

// ---------------------------------------------------------------------------------
static size_t al256(size_t x) { return (x + 255) / 256 * 256; }

struct OztLayout {
  int BN, Kp, Npad;
  size_t off_ey, off_ys, total;
};

static int ozt_bn(int nslice, int N) {
  if (nslice == 6) return N <= 64 ? 64 : (N <= 80 ? 80 : (N % 80 == 0 || N % 64 != 0 ? 80 : 64));
  return 64;
}

static OztLayout ozt_layout(int N, int K, int nslice) {
  OztLayout L;
  L.BN = ozt_bn(nslice, N);
  L.Kp = (K + OZT_BK - 1) / OZT_BK * OZT_BK;
  L.Npad = (N + L.BN - 1) / L.BN * L.BN;
  L.off_ey = 256;
  L.off_ys = al256(L.off_ey + (size_t)L.Npad * 4);
  L.total = al256(L.off_ys + (size_t)L.Npad * nslice * L.Kp * 2);
  return L;
}

typedef CUresult (*PcgEncodeTiled)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                    const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                    CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static int get_encode_tiled(PcgEncodeTiled* fn) {
  static PcgEncodeTiled cached = nullptr;
  if (!cached) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !p) {
      pcg_set_error("cuTensorMapEncodeTiled not available from the driver");
      return PCG_ERR_CUDA;
    }
    cached = (PcgEncodeTiled)p;
  }
  *fn = cached;
  return PCG_OK;
}

template <int NS, int BN>
static int ozt_run(long long M, int N, int K, const double* X, long long ldx, const double* Y, long long sYk, long long sYn,
                   double* C, long long sCm, long long sCn, int accumulate, char* ws, const OztLayout& L,
                   cudaStream_t s) {
  using Cfg = OztCfg<NS, BN>;
  int* err = (int*)ws;
  int* ey = (int*)(ws + L.off_ey);
  __nv_bfloat16* ys = (__nv_bfloat16*)(ws + L.off_ys);
  k_ozt_split_y<NS><<<(L.Npad + 7) / 8, 256, 0, s>>>(Y, sYk, sYn, K, N, L.Npad, L.Kp, ys, ey);
  PCG_CUDA(cudaGetLastError());
  // Y slices as a 2-D tensor [NS * Npad rows][Kp columns] of BF16; boxes of 32 columns
  // (64 bytes, the swizzle span) by BN rows; k0 is a multiple of 32, so every copy
  // starts on a 64-byte boundary
  PcgEncodeTiled encode;
  if (int rc = get_encode_tiled(&encode)) return rc;
  CUtensorMap ymap;
  const cuuint64_t gdim[2] = {(cuuint64_t)L.Kp, (cuuint64_t)NS * L.Npad};
  const cuuint64_t gstride[1] = {(cuuint64_t)L.Kp * 2};
  const cuuint32_t box[2] = {OZT_BK, BN};
  const cuuint32_t estr[2] = {1, 1};
  if (encode(&ymap, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (void*)ys, gdim, gstride, box, estr,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS) {
    pcg_set_error("pcg_ozaki_gemm_tc: cuTensorMapEncodeTiled rejected the Y slice layout");
    return PCG_ERR_CUDA;
  }
  static bool attr_set[64];
  int dev = 0;
  PCG_CUDA(cudaGetDevice(&dev));
  if (dev >= 0 && dev < 64 && !attr_set[dev]) {
    PCG_CUDA(cudaFuncSetAttribute(k_ozt_gemm<NS, BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, Cfg::SMEM));
    attr_set[dev] = true;
  }
  const long long blocks = (long long)(L.Npad / BN) * ((M + OZT_BM - 1) / OZT_BM);
  k_ozt_gemm<NS, BN><<<(unsigned)blocks, OZT_THREADS, Cfg::SMEM, s>>>(M, N, K, L.Kp, L.Npad, X, ldx, ymap, ey, C, sCm,
                                                                    sCn, accumulate, err);
  PCG_CUDA(cudaGetLastError());
  return PCG_OK;
}

extern "C" size_t pcg_ozaki_tc_workspace(int N, int K, int nslice) {
  if (N < 1 || K < 1 || (nslice != 6 && nslice != 7)) return 0;
  return ozt_layout(N, K, nslice).total;
}

extern "C" int pcg_ozaki_gemm_tc(long long M, int N, int K, const double* X, long long ldx, const double* Y, long long sYk,
                                 long long sYn, double* C, long long sCm, long long sCn, int nslice, int accumulate,
                                 void* workspace, size_t ws_bytes, void* stream) {
  if (M < 1 || N < 1 || K < 1 || !X || !Y || !C || ldx < K) {
    pcg_set_error("pcg_ozaki_gemm_tc: bad arguments");
    return PCG_ERR_ARG;
  }
  if (nslice != 6 && nslice != 7) {
    pcg_set_error("pcg_ozaki_gemm_tc: nslice must be 6 or 7");
    return PCG_ERR_UNSUPPORTED;
  }
  if ((long long)K * (nslice + 2) >= 4096) {
    pcg_set_error("pcg_ozaki_gemm_tc: K too large for exact FP32 level sums (need K * (nslice + 2) < 4096)");
    return PCG_ERR_UNSUPPORTED;
  }
  const OztLayout L = ozt_layout(N, K, nslice);
  if ((M + OZT_BM - 1) / OZT_BM * (long long)(L.Npad / L.BN) >= (1ll << 31)) {
    pcg_set_error("pcg_ozaki_gemm_tc: M too large for one launch");
    return PCG_ERR_UNSUPPORTED;
  }
  if (!workspace || ws_bytes < L.total || ((size_t)workspace & 255)) {
    pcg_set_error("pcg_ozaki_gemm_tc: workspace missing, too small or not 256-byte aligned (query pcg_ozaki_tc_workspace)");
    return PCG_ERR_CAPACITY;
  }
  cudaStream_t s = (cudaStream_t)stream;
  char* ws = (char*)workspace;
  PCG_CUDA(cudaMemsetAsync(ws, 0, 4, s));
  if (nslice == 7) return ozt_run<7, 64>(M, N, K, X, ldx, Y, sYk, sYn, C, sCm, sCn, accumulate, ws, L, s);
  if (L.BN == 80) return ozt_run<6, 80>(M, N, K, X, ldx, Y, sYk, sYn, C, sCm, sCn, accumulate, ws, L, s);
  return ozt_run<6, 64>(M, N, K, X, ldx, Y, sYk, sYn, C, sCm, sCn, accumulate, ws, L, s);
}

// Error flag of the last pcg_ozaki_gemm_tc call that used this workspace (0: no CTA
// gave up on a wait); synchronises the stream.
extern "C" int pcg_ozaki_tc_status(const void* workspace, void* stream) {
  int h = 0;
  PCG_CUDA(cudaMemcpyAsync(&h, workspace, 4, cudaMemcpyDeviceToHost, (cudaStream_t)stream));
  PCG_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
  return h;
}
