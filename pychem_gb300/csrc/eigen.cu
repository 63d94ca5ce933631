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
// small-molecule SCF).  T = float (n <= 334) keeps packed A and V in shared memory
// too, V's rows spread over as many CTAs per matrix as that takes (two at n = 208,
// eight at n = 298); the caller refines the float result in FP64 (Ogita-Aishima
// iteration, pychem_gb300/eigen.py), so the O(n^3) rotation work runs on the FP32
// pipe.
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
//
// One matrix may be spread over `split` CTAs: every CTA holds the whole packed A and
// applies the same rotations to it (the same arithmetic in the same order, so the
// copies stay identical and need no communication), and rows [r0, r1) of V, in shared
// memory; rotations act on each row of V separately.  That keeps V out of global
// memory for n up to 334 in FP32.  With use_tab, the (k, k2) pair of every 2x2 block
// is read from a table in shared memory (after V) instead of being decoded with a
// square root per block and round.  Rotations that are the identity (a_pq = 0) skip
// their updates.
template <typename T>
__global__ void __launch_bounds__(1024) k_jacobi(int n, int m, int split, int rows_per, const double* __restrict__ Ain,
                                                 long long sA, T* __restrict__ Vg, long long sV,
                                                 const T* __restrict__ V0, double* __restrict__ w, long long sw,
                                                 int max_sweeps, double tol, int* __restrict__ info, int use_tab) {
  extern __shared__ unsigned char smem_raw[];
  T* A = (T*)smem_raw;
  const int ntri = m * (m + 1) / 2;
  const int b = blockIdx.x / split, part = blockIdx.x % split;
  const int r0 = part * rows_per, r1 = min(m, r0 + rows_per), nrow = max(0, r1 - r0);
  T* V = A + ((ntri + 1) & ~1);                      // rows r0..r1 of V (nrow x m)
  unsigned* tab = (unsigned*)(V + (((size_t)rows_per * m + 1) & ~(size_t)1));
  constexpr int HMAX = 176;                          // m / 2 <= 167
  __shared__ T cs[HMAX], sn[HMAX];
  __shared__ int pp[HMAX], qq[HMAX];
  __shared__ double red0[32], red1[32];
  __shared__ int stop;
  const double* Ab = Ain + (size_t)b * sA;
  const int nt = blockDim.x, tid = threadIdx.x;
  for (int idx = tid; idx < ntri; idx += nt) {
    int i = (int)((sqrtf(8.0f * idx + 1.0f) - 1.0f) * 0.5f);
    while (tri(i + 1, 0) <= idx) ++i;
    while (tri(i, 0) > idx) --i;
    const int j = idx - tri(i, 0);
    A[idx] = (i < n && j < n) ? (T)Ab[(size_t)i * n + j] : (T)0;
  }
  for (int idx = tid; idx < nrow * m; idx += nt) {
    const int i = r0 + idx / m, j = idx % m;
    T v = (T)(i == j);
    if (V0 && i < n && j < n) v = V0[(size_t)b * sV + (size_t)i * m + j];
    V[idx] = v;
  }
  if (tid == 0) stop = 0;
  const int h = m / 2;
  const int nblk = h * (h + 1) / 2;
  if (use_tab)
    for (int k = tid; k < h; k += nt)
      for (int k2 = 0; k2 <= k; ++k2) tab[k * (k + 1) / 2 + k2] = ((unsigned)k << 16) | (unsigned)k2;
  __syncthreads();
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
      for (int it = tid; it < nblk + nrow * h; it += nt) {
        if (it < nblk) {
          int k, k2;  // k >= k2
          if (use_tab) {
            const unsigned e = tab[it];
            k = (int)(e >> 16); k2 = (int)(e & 0xFFFFu);
          } else {
            k = (int)((sqrtf(8.0f * it + 1.0f) - 1.0f) * 0.5f);
            while ((k + 1) * (k + 2) / 2 <= it) ++k;
            while (k * (k + 1) / 2 > it) --k;
            k2 = it - k * (k + 1) / 2;
          }
          const int p = pp[k], q = qq[k], p2 = pp[k2], q2 = qq[k2];
          const T c = cs[k], s = sn[k], c2 = cs[k2], s2 = sn[k2];
          if (s == (T)0 && s2 == (T)0) continue;   // both rotations the identity
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
          const int i = t / h, k = t % h;            // local row i of V
          const T c = cs[k], s = sn[k];
          if (s == (T)0) continue;
          const int p = pp[k], q = qq[k];
          const T vp = V[i * m + p], vq = V[i * m + q];
          V[i * m + p] = c * vp - s * vq;
          V[i * m + q] = s * vp + c * vq;
        }
      }
      __syncthreads();
    }
  }
  if (part == 0) {
    for (int i = tid; i < n; i += nt) w[(size_t)b * sw + i] = (double)A[tri(i, i)];
    if (tid == 0 && info) info[b] = sweep;
  }
  for (int idx = tid; idx < nrow * m; idx += nt) Vg[(size_t)b * sV + (size_t)r0 * m + idx] = V[idx];
}

// shared-memory plan of one launch: how many CTAs share a matrix, rows of V per CTA,
// whether the block table fits, and the dynamic bytes
template <typename T>
static bool jacobi_plan(int m, int& split, int& rows_per, int& tab, size_t& bytes) {
  const size_t limit = 232448 - 5120;                // 227 KB less the static tables
  const size_t a_bytes = (size_t)((m * (m + 1) / 2 + 1) & ~1) * sizeof(T);
  const size_t tab_bytes = (size_t)(m / 2) * (m / 2 + 1) / 2 * sizeof(unsigned);
  for (split = 1; split <= m; ++split) {
    rows_per = (m + split - 1) / split;
    const size_t v_bytes = (size_t)(((size_t)rows_per * m + 1) & ~(size_t)1) * sizeof(T);
    if (a_bytes + v_bytes <= limit) {
      tab = a_bytes + v_bytes + tab_bytes <= limit;
      bytes = a_bytes + v_bytes + (tab ? tab_bytes : 0);
      return true;
    }
  }
  return false;
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
  // above n = 64 one CTA per SM is resident anyway (shared memory): 1024 threads
  const int threads = m <= 32 ? 128 : (m <= 64 ? 256 : 1024);
  int split = 1, rows_per = m, tab = 0;
  size_t bytes = 0;
  if (!fp32) {
    if (m / 2 > 68 || !jacobi_plan<double>(m, split, rows_per, tab, bytes) || split != 1) {
      pcg_set_error("pcg_jacobi_eigh: FP64 variant needs n <= 136");
      return PCG_ERR_UNSUPPORTED;
    }
    PCG_CUDA(cudaFuncSetAttribute(k_jacobi<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    k_jacobi<double><<<batch, threads, bytes, s>>>(n, m, 1, m, A, sA, (double*)V, sV, (const double*)V0, w, sw,
                                                   max_sweeps, tol, info, tab);
  } else {
    if (m / 2 > 167 || !jacobi_plan<float>(m, split, rows_per, tab, bytes)) {
      pcg_set_error("pcg_jacobi_eigh: FP32 variant needs n <= 334");
      return PCG_ERR_UNSUPPORTED;
    }
    if ((long long)batch * split > 0x7fffffffLL) { pcg_set_error("pcg_jacobi_eigh: batch too large"); return PCG_ERR_ARG; }
    PCG_CUDA(cudaFuncSetAttribute(k_jacobi<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    k_jacobi<float><<<batch * split, threads, bytes, s>>>(n, m, split, rows_per, A, sA, (float*)V, sV,
                                                          (const float*)V0, w, sw, max_sweeps, tol, info, tab);
  }
  PCG_CUDA(cudaGetLastError());
  return PCG_OK;
}
