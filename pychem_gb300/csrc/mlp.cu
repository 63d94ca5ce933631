// Kernels of the learned initial-guess network: dense layers with BF16 weights and
// FP32 accumulation, SiLU activation, masked squared-error loss and Adam.
//
// One tiled GEMM serves the forward pass and both backward products:
//   C[m][n] (+)= sum_k A(m, k) B(k, n),  A(m, k) = A[m*sam + k*sak] (FP32),
//   B(k, n) = B[k*sbk + n*sbn] (FP32 or BF16), C row-major with ldc,
// with an optional epilogue Z = C + bias, C = silu(Z).  64x64 output tiles, K in
// steps of 16 through shared memory, 256 threads with a 4x4 micro-tile each.
#include <cuda_bf16.h>
#include <math.h>

#include "../../include/pychem_gb300.h"
#include "common.cuh"
#include "pcg_internal.h"

#define MT 64
#define KT 16

template <typename TB>
__device__ __forceinline__ float ldb_(const TB* p) { return (float)*p; }
template <>
__device__ __forceinline__ float ldb_<__nv_bfloat16>(const __nv_bfloat16* p) { return __bfloat162float(*p); }

__device__ __forceinline__ float silu(float z) { return z / (1.0f + __expf(-z)); }
__device__ __forceinline__ float dsilu(float z) {
  const float s = 1.0f / (1.0f + __expf(-z));
  return s * (1.0f + z * (1.0f - s));
}

template <typename TB>
__global__ void __launch_bounds__(256) k_gemm(int M, int N, int K, const float* __restrict__ A, long long sam,
                                              long long sak, const TB* __restrict__ B, long long sbk, long long sbn,
                                              float* __restrict__ C, int ldc, int accumulate,
                                              const float* __restrict__ bias, float* __restrict__ Z, int act) {
  __shared__ float As[KT][MT + 4];
  __shared__ float Bs[KT][MT + 4];
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  const int m0 = blockIdx.y * MT, n0 = blockIdx.x * MT;
  float acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.0f;
  for (int k0 = 0; k0 < K; k0 += KT) {
    for (int idx = threadIdx.x; idx < KT * MT; idx += 256) {
      // A tile: consecutive threads along m when sam == 1, else along k
      int kk, mm;
      if (sam == 1) { mm = idx % MT; kk = idx / MT; } else { kk = idx % KT; mm = idx / KT; }
      const int m = m0 + mm, k = k0 + kk;
      As[kk][mm] = (m < M && k < K) ? A[(long long)m * sam + (long long)k * sak] : 0.0f;
      int kb, nn;
      if (sbn == 1) { nn = idx % MT; kb = idx / MT; } else { kb = idx % KT; nn = idx / KT; }
      const int n = n0 + nn, k2 = k0 + kb;
      Bs[kb][nn] = (n < N && k2 < K) ? ldb_<TB>(B + (long long)k2 * sbk + (long long)n * sbn) : 0.0f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < KT; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int m = m0 + ty * 4 + i;
    if (m >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int n = n0 + tx * 4 + j;
      if (n >= N) continue;
      float v = acc[i][j];
      float* c = C + (long long)m * ldc + n;
      if (accumulate) v += *c;
      if (bias) v += bias[n];
      if (Z) Z[(long long)m * ldc + n] = v;
      if (act) v = silu(v);
      *c = v;
    }
  }
}

// G = dY * silu'(Z) elementwise (in place on dY)
__global__ void k_dsilu(long long n, float* __restrict__ dY, const float* __restrict__ Z) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dY[i] *= dsilu(Z[i]);
}

// column sums: db[n] = sum_m G[m][n]
__global__ void k_colsum(int M, int N, const float* __restrict__ G, float* __restrict__ db) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  float s = 0.0f;
  for (int m = 0; m < M; ++m) s += G[(long long)m * N + n];
  db[n] = s;
}

// masked squared error: loss partial sums and dY = 2 (Y - T) mask / count
__global__ void k_mse(long long n, const float* __restrict__ Y, const float* __restrict__ T,
                      const float* __restrict__ mask, float inv_count, float* __restrict__ dY,
                      float* __restrict__ loss) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  float l = 0.0f;
  if (i < n) {
    const float d = (Y[i] - T[i]) * mask[i];
    dY[i] = 2.0f * d * inv_count;
    l = d * d * inv_count;
  }
  for (int o = 16; o > 0; o >>= 1) l += __shfl_down_sync(0xffffffffu, l, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, l);
}

// Adam on FP32 master weights, refreshing the BF16 copy used by the GEMMs
__global__ void k_adam(long long n, float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, __nv_bfloat16* __restrict__ wb, float lr, float b1, float b2, float eps,
                       float c1, float c2) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.0f - b1) * gi;
  const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float wi = w[i] - lr * (mi * c1) / (sqrtf(vi * c2) + eps);
  w[i] = wi;
  if (wb) wb[i] = __float2bfloat16_rn(wi);
}

extern "C" int pcg_mlp_gemm(int M, int N, int K, const float* A, long long sam, long long sak, const void* B,
                            int b_bf16, long long sbk, long long sbn, float* C, int ldc, int accumulate,
                            const float* bias, float* Z, int act, void* stream) {
  if (M < 1 || N < 1 || K < 1 || !A || !B || !C) { pcg_set_error("pcg_mlp_gemm: bad arguments"); return PCG_ERR_ARG; }
  dim3 grid((N + MT - 1) / MT, (M + MT - 1) / MT);
  cudaStream_t s = (cudaStream_t)stream;
  if (b_bf16)
    k_gemm<__nv_bfloat16><<<grid, 256, 0, s>>>(M, N, K, A, sam, sak, (const __nv_bfloat16*)B, sbk, sbn, C, ldc,
                                               accumulate, bias, Z, act);
  else
    k_gemm<float><<<grid, 256, 0, s>>>(M, N, K, A, sam, sak, (const float*)B, sbk, sbn, C, ldc, accumulate, bias, Z,
                                       act);
  PCG_CUDA(cudaGetLastError());
  return PCG_OK;
}

extern "C" int pcg_mlp_dsilu(long long n, float* dY, const float* Z, void* stream) {
  k_dsilu<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(n, dY, Z);
  PCG_CUDA(cudaGetLastError());
  return PCG_OK;
}

extern "C" int pcg_mlp_colsum(int M, int N, const float* G, float* db, void* stream) {
  k_colsum<<<(N + 127) / 128, 128, 0, (cudaStream_t)stream>>>(M, N, G, db);
  PCG_CUDA(cudaGetLastError());
  return PCG_OK;
}

extern "C" int pcg_mlp_mse(long long n, const float* Y, const float* T, const float* mask, float inv_count,
                           float* dY, float* loss, void* stream) {
  k_mse<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(n, Y, T, mask, inv_count, dY, loss);
  PCG_CUDA(cudaGetLastError());
  return PCG_OK;
}

extern "C" int pcg_mlp_adam(long long n, float* w, const float* g, float* m, float* v, void* w_bf16, float lr,
                            float b1, float b2, float eps, int step, void* stream) {
  const float c1 = 1.0f / (1.0f - powf(b1, (float)step)), c2 = 1.0f / (1.0f - powf(b2, (float)step));
  k_adam<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(n, w, g, m, v, (__nv_bfloat16*)w_bf16, lr,
                                                                        b1, b2, eps, c1, c2);
  PCG_CUDA(cudaGetLastError());
  return PCG_OK;
}
