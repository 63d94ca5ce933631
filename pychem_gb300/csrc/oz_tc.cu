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
//    FP64 from global memory and split on the fly: eight producer warps load a 128-row
//    by 32-column chunk, cut it into NS digit slices and store them BF16, K-major and
//    64-byte swizzled, straight into the shared-memory operand tiles (no BF16 copy of
//    X in global memory).  The exponent of each row comes from a first pass over the
//    CTA's rows (the re-read is served by L2).
//  * Y, the small operand (C_occ or C_vir: a few hundred columns), is split once by
//    k_ozt_split_y into K-major BF16 slices in the caller's workspace and copied tile by
//    tile into shared memory by the same producer warps.
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
#include <cuda_bf16.h>
#include <stdio.h>

#include "../../include/pychem_gb300.h"
#include "common.cuh"
#include "ozaki_common.cuh"
#include "pcg_internal.h"
#include "umma.cuh"

#define OZT_BM 128
#define OZT_BK 32
#define OZT_PROD_WARPS 8
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

// Y slices: ys[(n * NS + p) * Kp + k] (BF16, zero for k >= K and n >= N), ey[n]: one
// warp per column n, lanes over k.
template <int NS>
__global__ void k_ozt_split_y(const double* __restrict__ Y, long long sYk, long long sYn, int K, int N, int Npad,
                              int Kp, __nv_bfloat16* __restrict__ ys, int* __restrict__ ey) {
  const int n = blockIdx.x * 8 + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (n >= Npad) return;
  __nv_bfloat16* out = ys + (size_t)n * NS * Kp;
  if (n >= N) {
    for (int i = lane; i < NS * Kp; i += 32) out[i] = __float2bfloat16(0.0f);
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
    for (int p = 0; p < NS; ++p) out[(size_t)p * Kp + k] = __int2bfloat16_rn(d[p]);
  }
}

template <int NS, int BN>
__global__ void __launch_bounds__(OZT_THREADS, 1)
    k_ozt_gemm(int M, int N, int K, int Kp, const double* __restrict__ X, long long ldx,
               const __nv_bfloat16* __restrict__ ys, const int* __restrict__ ey, double* __restrict__ C, long long sCm,
               long long sCn, int accumulate, int* __restrict__ err) {
  using Cfg = OztCfg<NS, BN>;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* sm = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint8_t* tiles = sm;                                        // [stage][X slices | Y slices]
  uint64_t* bars = (uint64_t*)(sm + 2 * Cfg::STAGE);          // full[2], empty[2], done, drain
  uint32_t* tmem_slot = (uint32_t*)(bars + 6);
  volatile int* abort_s = (volatile int*)(tmem_slot + 1);
  int* ex_s = (int*)(tmem_slot + 4);                           // 128 row exponent fields

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.y * OZT_BM;
  const int n0 = blockIdx.x * BN;
  const int nchunk = Kp / OZT_BK;

  if (threadIdx.x == 0) {
    for (int i = 0; i < 2; ++i) { mbar_init(&bars[i], OZT_PROD); mbar_init(&bars[2 + i], 1); }
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
    // ---- exponents of the CTA's 128 rows of X
    for (int r = warp; r < OZT_BM; r += OZT_PROD_WARPS) {
      const int m = m0 + r;
      unsigned long long mx = 0;
      if (m < M)
        for (int k = lane; k < K; k += 32) mx = max(mx, oz_absbits(__ldg(X + (long long)m * ldx + k)));
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
      if (lane == 0) ex_s[r] = (int)(mx >> 52);
    }
    asm volatile("bar.sync 1, %0;" ::"r"(OZT_PROD));
    const int t = threadIdx.x;
    bool ok = true;
    for (int c = 0; c < nchunk && ok; ++c) {
      const int st = c & 1;
      if (c >= 2 && !mbar_wait(&bars[2 + st], ((c >> 1) + 1) & 1, OZT_WAIT, abort_s)) { ok = false; break; }
      uint8_t* xt = tiles + st * Cfg::STAGE;
      uint8_t* yt = xt + NS * Cfg::XT;
      const int k0 = c * OZT_BK;
      // X: 128 rows x 4 groups of 8 columns; item i -> row i / 4, group i % 4
#pragma unroll 1
      for (int i = t; i < OZT_BM * 4; i += OZT_PROD) {
        const int r = i >> 2, g = i & 3, m = m0 + r;
        const int kb = k0 + 8 * g;
        double v[8];
        if (m < M) {
          const double* src = X + (long long)m * ldx + kb;
#pragma unroll
          for (int j = 0; j < 8; ++j) v[j] = (kb + j < K) ? __ldg(src + j) : 0.0;
        } else {
#pragma unroll
          for (int j = 0; j < 8; ++j) v[j] = 0.0;
        }
        const int emax = ex_s[r];
        int d[8][NS];
#pragma unroll
        for (int j = 0; j < 8; ++j) oz_digits<NS>(v[j], emax, d[j]);
        const uint32_t off = sw64_offset(r, g);
#pragma unroll
        for (int p = 0; p < NS; ++p) {
          uint32_t w[4];
#pragma unroll
          for (int h = 0; h < 4; ++h) {
            __nv_bfloat162 b2 = __halves2bfloat162(__int2bfloat16_rn(d[2 * h][p]), __int2bfloat16_rn(d[2 * h + 1][p]));
            w[h] = *(uint32_t*)&b2;
          }
          *(uint4*)(xt + p * Cfg::XT + off) = make_uint4(w[0], w[1], w[2], w[3]);
        }
      }
      // Y: NS slices x BN rows x 4 chunks of 16 bytes
#pragma unroll 1
      for (int i = t; i < NS * BN * 4; i += OZT_PROD) {
        const int ch = i & 3, n = (i >> 2) % BN, p = (i >> 2) / BN;
        const uint4 q = __ldg((const uint4*)(ys + ((size_t)(n0 + n) * NS + p) * Kp + k0) + ch);
        *(uint4*)(yt + p * Cfg::YT + sw64_offset(n, ch)) = q;
      }
      fence_proxy_async_smem();
      mbar_arrive(&bars[st]);
    }
    if (!ok) { *abort_s = 1; atomicExch(err, 1); }
    // ---- epilogue: wait for the last MMAs, combine the levels, write C
    if (ok && mbar_wait(&bars[4], 0, OZT_WAIT, abort_s)) {
      tc_fence_after();
      const int lg = warp & 3, half = warp >> 2;
      const int r = 32 * lg + lane, m = m0 + r;
      const int emax = ex_s[r];
      const int ex = (emax ? emax - 1022 : 0) - OZ_BETA * (NS + 1);
      const uint32_t trow = tmem + ((uint32_t)(32 * lg) << 16);
#pragma unroll 1
      for (int cb = half * (BN / 2); cb < (half + 1) * (BN / 2); cb += 8) {
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
            double* cp = C + (long long)m * sCm + (long long)n * sCn;
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
      if (!mbar_wait(&bars[st], (c >> 1) & 1, OZT_WAIT, abort_s)) { ok = false; break; }
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

template <int NS, int BN>
static int ozt_run(int M, int N, int K, const double* X, long long ldx, const double* Y, long long sYk, long long sYn,
                   double* C, long long sCm, long long sCn, int accumulate, char* ws, const OztLayout& L,
                   cudaStream_t s) {
  using Cfg = OztCfg<NS, BN>;
  int* err = (int*)ws;
  int* ey = (int*)(ws + L.off_ey);
  __nv_bfloat16* ys = (__nv_bfloat16*)(ws + L.off_ys);
  k_ozt_split_y<NS><<<(L.Npad + 7) / 8, 256, 0, s>>>(Y, sYk, sYn, K, N, L.Npad, L.Kp, ys, ey);
  PCG_CUDA(cudaGetLastError());
  static bool attr_set[64];
  int dev = 0;
  PCG_CUDA(cudaGetDevice(&dev));
  if (dev >= 0 && dev < 64 && !attr_set[dev]) {
    PCG_CUDA(cudaFuncSetAttribute(k_ozt_gemm<NS, BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, Cfg::SMEM));
    attr_set[dev] = true;
  }
  dim3 grid(L.Npad / BN, (M + OZT_BM - 1) / OZT_BM);
  k_ozt_gemm<NS, BN><<<grid, OZT_THREADS, Cfg::SMEM, s>>>(M, N, K, L.Kp, X, ldx, ys, ey, C, sCm, sCn, accumulate,
                                                         err);
  PCG_CUDA(cudaGetLastError());
  return PCG_OK;
}

extern "C" size_t pcg_ozaki_tc_workspace(int N, int K, int nslice) {
  if (N < 1 || K < 1 || (nslice != 6 && nslice != 7)) return 0;
  return ozt_layout(N, K, nslice).total;
}

extern "C" int pcg_ozaki_gemm_tc(int M, int N, int K, const double* X, long long ldx, const double* Y, long long sYk,
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
  if ((long long)(M + OZT_BM - 1) / OZT_BM > 65535) {
    pcg_set_error("pcg_ozaki_gemm_tc: M too large for one launch (at most 65535 * 128 rows)");
    return PCG_ERR_UNSUPPORTED;
  }
  const OztLayout L = ozt_layout(N, K, nslice);
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
