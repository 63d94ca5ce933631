// Batched symmetric eigensolver: parallel cyclic Jacobi, one CTA per matrix.
//
// Method: two-sided Jacobi rotations B = J^T A J (Golub & Van Loan, Matrix
// Computations, 4th ed., Alg. 8.5.2 sym.schur2 for the rotation), applied to n/2
// disjoint index pairs at a time in the round-robin ("circle method") order, so one
// sweep is n-1 rounds of n/2 independent rotations.  Rows of A are updated for all
// pairs, then columns of A and of V; the sweep loop stops when the off-diagonal
// Frobenius norm falls below tol times the total norm.
//
// T = double keeps A (packed) and V in shared memory (n <= 136; used by the batched
// small-molecule SCF).  T = float keeps packed A in shared memory and V in global
// memory (n <= 334 with 227 KB of shared memory); the caller refines the float result in FP64
// (Ogita-Aishima iteration, pychem_gb300/eigen.py), so the O(n^3) rotation work runs
// on the FP32 pipe.
#include <math.h>

#include "../../include/pychem_gb300.h"
#include "common.cuh"
#include "pcg_internal.h"

template <typename T>
__device__ __forceinline__ void rot_params(T app, T aqq, T apq, T& c, T& s) {
  if (apq == (T)0) { c = (T)1; s = (T)0; return; }
  const T tau = (aqq - app) / ((T)2 * apq);
  T t;
  if (fabs(tau) > (T)1e18) t = (T)0.5 / tau;
  else t = (tau >= (T)0 ? (T)1 : (T)-1) / (fabs(tau) + sqrt((T)1 + tau * tau));
  c = (T)1 / sqrt((T)1 + t * t);
  s = t * c;
}

__device__ __forceinline__ int tri(int i, int j) {  // packed lower triangle, i >= j
  return i * (i + 1) / 2 + j;
}
__device__ __forceinline__ int sym(int i, int j) { return i >= j ? tri(i, j) : tri(j, i); }

// A is held as a packed lower triangle in shared memory.  Each round first computes
// the n/2 rotations, then transforms every 2x2 block (pair k rows, pair k' columns,
// k >= k') as B' = J_k^T B J_k' -- blocks are disjoint, so one pass suffices -- and
// the rows of V as V J.
template <typename T, bool V_SMEM>
__global__ void k_jacobi(int n, int m, const double* __restrict__ Ain, long long sA, T* __restrict__ Vg, long long sV,
                         const T* __restrict__ V0, double* __restrict__ w, long long sw, int max_sweeps, double tol,
                         int* __restrict__ info) {
  extern __shared__ unsigned char smem_raw[];
  T* A = (T*)smem_raw;
  const int ntri = m * (m + 1) / 2;
  T* V = V_SMEM ? A + ((ntri + 1) & ~1) : Vg + (size_t)blockIdx.x * sV;
  // rotation tables: m/2 entries (m <= 136 for the shared-memory variant, whose
  // dynamic part then leaves room for only a few KB of static shared memory)
  constexpr int HMAX = V_SMEM ? 128 : 512;
  __shared__ T cs[HMAX], sn[HMAX];
  __shared__ int pp[HMAX], qq[HMAX];
  __shared__ double red0[32], red1[32];
  __shared__ int stop;
  const int b = blockIdx.x;
  const double* Ab = Ain + (size_t)b * sA;
  const int nt = blockDim.x, tid = threadIdx.x;
  for (int idx = tid; idx < ntri; idx += nt) {
    int i = (int)((sqrtf(8.0f * idx + 1.0f) - 1.0f) * 0.5f);
    while (tri(i + 1, 0) <= idx) ++i;
    while (tri(i, 0) > idx) --i;
    const int j = idx - tri(i, 0);
    A[idx] = (i < n && j < n) ? (T)Ab[(size_t)i * n + j] : (T)0;
  }
  for (int idx = tid; idx < m * m; idx += nt) {
    const int i = idx / m, j = idx % m;
    T v = (T)(i == j);
    if (V0 && i < n && j < n) v = V0[(size_t)b * sV + idx];
    V[idx] = v;
  }
  if (tid == 0) stop = 0;
  __syncthreads();
  const int h = m / 2;
  const int nblk = h * (h + 1) / 2;
  int sweep = 0;
  for (; sweep < max_sweeps; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int idx = tid; idx < ntri; idx += nt) {
      const double a = (double)A[idx];
      int i = (int)((sqrtf(8.0f * idx + 1.0f) - 1.0f) * 0.5f);
      while (tri(i + 1, 0) <= idx) ++i;
      while (tri(i, 0) > idx) --i;
      const bool diag = (idx - tri(i, 0)) == i;
      tot += diag ? a * a : 2.0 * a * a;
      if (!diag) off += 2.0 * a * a;
    }
    for (int o = 16; o > 0; o >>= 1) {
      off += __shfl_down_sync(0xffffffffu, off, o);
      tot += __shfl_down_sync(0xffffffffu, tot, o);
    }
    if ((tid & 31) == 0) { red0[tid >> 5] = off; red1[tid >> 5] = tot; }
    __syncthreads();
    if (tid == 0) {
      double o2 = 0.0, t2 = 0.0;
      for (int k = 0; k < (nt + 31) / 32; ++k) { o2 += red0[k]; t2 += red1[k]; }
      stop = (o2 <= tol * tol * t2) ? 1 : 0;
    }
    __syncthreads();
    if (stop) break;
    for (int r = 0; r < m - 1; ++r) {
      for (int k = tid; k < h; k += nt) {
        // circle method: position 0 fixed, positions 1..m-1 rotate by r
        const int a0 = (k == 0) ? 0 : 1 + (k - 1 + r) % (m - 1);
        const int a1 = 1 + (m - 2 - k + r) % (m - 1);
        const int p = min(a0, a1), q = max(a0, a1);
        T c, s;
        rot_params(A[tri(p, p)], A[tri(q, q)], A[tri(q, p)], c, s);
        pp[k] = p; qq[k] = q; cs[k] = c; sn[k] = s;
      }
      __syncthreads();
      for (int it = tid; it < nblk + m * h; it += nt) {
        if (it < nblk) {
          int k = (int)((sqrtf(8.0f * it + 1.0f) - 1.0f) * 0.5f);
          while ((k + 1) * (k + 2) / 2 <= it) ++k;
          while (k * (k + 1) / 2 > it) --k;
          const int k2 = it - k * (k + 1) / 2;  // k >= k2
          const int p = pp[k], q = qq[k], p2 = pp[k2], q2 = qq[k2];
          const T c = cs[k], s = sn[k], c2 = cs[k2], s2 = sn[k2];
          if (k == k2) {
            const T app = A[tri(p, p)], aqq = A[tri(q, q)], apq = A[tri(q, p)];
            // J^T [[app, apq], [apq, aqq]] J with the rotation that zeroes apq
            A[tri(p, p)] = c * c * app - (T)2 * c * s * apq + s * s * aqq;
            A[tri(q, q)] = s * s * app + (T)2 * c * s * apq + c * c * aqq;
            A[tri(q, p)] = (T)0;
          } else {
            const int ipp = sym(p, p2), ipq = sym(p, q2), iqp = sym(q, p2), iqq = sym(q, q2);
            const T b00 = A[ipp], b01 = A[ipq], b10 = A[iqp], b11 = A[iqq];
            // rows: J_k^T B
            const T r00 = c * b00 - s * b10, r01 = c * b01 - s * b11;
            const T r10 = s * b00 + c * b10, r11 = s * b01 + c * b11;
            // columns: (J_k^T B) J_k2
            A[ipp] = c2 * r00 - s2 * r01;
            A[ipq] = s2 * r00 + c2 * r01;
            A[iqp] = c2 * r10 - s2 * r11;
            A[iqq] = s2 * r10 + c2 * r11;
          }
        } else {
          const int t = it - nblk;
          const int i = t / h, k = t % h;
          const int p = pp[k], q = qq[k];
          const T c = cs[k], s = sn[k];
          const T vp = V[i * m + p], vq = V[i * m + q];
          V[i * m + p] = c * vp - s * vq;
          V[i * m + q] = s * vp + c * vq;
        }
      }
      __syncthreads();
    }
  }
  for (int i = tid; i < n; i += nt) w[(size_t)b * sw + i] = (double)A[tri(i, i)];
  if (V_SMEM)
    for (int idx = tid; idx < m * m; idx += nt) Vg[(size_t)b * sV + idx] = V[idx];
  if (tid == 0 && info) info[b] = sweep;
}

extern "C" int pcg_jacobi_eigh(int batch, int n, const double* A, double* w, void* V, int fp32, const void* V0,
                               int max_sweeps, double tol, int* info, void* stream) {
  if (batch < 1 || n < 1 || !A || !w || !V || max_sweeps < 1) {
    pcg_set_error("pcg_jacobi_eigh: bad arguments");
    return PCG_ERR_ARG;
  }
  const int m = n + (n & 1);
  if (m / 2 > 512 || m < 2) { pcg_set_error("pcg_jacobi_eigh: n out of range"); return PCG_ERR_UNSUPPORTED; }
  cudaStream_t s = (cudaStream_t)stream;
  {
    const cudaError_t prior = cudaGetLastError();
    if (prior != cudaSuccess) {
      pcg_set_cuda_error(prior, "an earlier asynchronous operation (reported on entry to pcg_jacobi_eigh)");
      return PCG_ERR_CUDA;
    }
  }
  const long long sA = (long long)n * n, sV = (long long)m * m, sw = n;
  if (!fp32) {
    const size_t smem = ((size_t)(m * (m + 1) / 2 + 1) / 2 * 2 + (size_t)m * m) * sizeof(double);
    if (smem > 220 * 1024 || m / 2 > 128) {
      pcg_set_error("pcg_jacobi_eigh: FP64 variant needs n <= 136");
      return PCG_ERR_UNSUPPORTED;
    }
    const int threads = m <= 32 ? 128 : 256;
    // opt in to the exact dynamic size: dynamic + static (3.5 KB) may exceed the
    // 48 KB default even when the dynamic part alone does not
    PCG_CUDA(cudaFuncSetAttribute(k_jacobi<double, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_jacobi<double, true><<<batch, threads, smem, s>>>(n, m, A, sA, (double*)V, sV, (const double*)V0, w, sw,
                                                         max_sweeps, tol, info);
  } else {
    // FP32: packed A and V both in shared memory while they fit (n <= 182), else V
    // in global memory (n <= 334)
    const size_t smem_v = ((size_t)(m * (m + 1) / 2 + 1) / 2 * 2 + (size_t)m * m) * sizeof(float);
    if (smem_v <= 200 * 1024 && m / 2 <= 128) {
      const int threads = m <= 32 ? 128 : 256;
      PCG_CUDA(cudaFuncSetAttribute(k_jacobi<float, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_v));
      k_jacobi<float, true><<<batch, threads, smem_v, s>>>(n, m, A, sA, (float*)V, sV, (const float*)V0, w, sw,
                                                            max_sweeps, tol, info);
    } else {
      const size_t smem = (size_t)m * (m + 1) / 2 * sizeof(float);
      if (smem > 220 * 1024) { pcg_set_error("pcg_jacobi_eigh: FP32 variant needs n <= 334"); return PCG_ERR_UNSUPPORTED; }
      PCG_CUDA(cudaFuncSetAttribute(k_jacobi<float, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      k_jacobi<float, false><<<batch, 1024, smem, s>>>(n, m, A, sA, (float*)V, sV, (const float*)V0, w, sw,
                                                        max_sweeps, tol, info);
    }
  }
  PCG_CUDA(cudaGetLastError());
  return PCG_OK;
}
