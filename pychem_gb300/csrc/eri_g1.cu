// ERI classes 6..13 (see eri_kernels.cuh); split for parallel compilation.
#include "eri_kernels.cuh"

int pcg_launch_eri_g1(int cls, const DevPairsExt& pr, const BoysTable& bt, const int2* tasks, int ntask,
                      double* store, int precision, cudaStream_t s) {
  const int threads = 128, blocks = (ntask + threads - 1) / threads;
  if (precision == 0) {
    switch (cls) {
      case 6: k_eri<Eri2000><<<blocks, threads, 0, s>>>(pr, bt, tasks, ntask, store); break;
      case 7: k_eri<Eri2010><<<blocks, threads, 0, s>>>(pr, bt, tasks, ntask, store); break;
      case 8: k_eri<Eri2011><<<blocks, threads, 0, s>>>(pr, bt, tasks, ntask, store); break;
      case 9: k_eri<Eri2020><<<blocks, threads, 0, s>>>(pr, bt, tasks, ntask, store); break;
      case 10: k_eri<Eri2100><<<blocks, threads, 0, s>>>(pr, bt, tasks, ntask, store); break;
      case 11: k_eri<Eri2110><<<blocks, threads, 0, s>>>(pr, bt, tasks, ntask, store); break;
      case 12: k_eri<Eri2111><<<blocks, threads, 0, s>>>(pr, bt, tasks, ntask, store); break;
      case 13: k_eri<Eri2120><<<blocks, threads, 0, s>>>(pr, bt, tasks, ntask, store); break;
      default: return PCG_ERR_ARG;
    }
  } else {
    switch (cls) {
      case 6: k_eri_f<Eri2000f><<<blocks, threads, 0, s>>>(pr, bt, tasks, ntask, store); break;
      case 7: k_eri_f<Eri2010f><<<blocks, threads, 0, s>>>(pr, bt, tasks, ntask, store); break;
      case 8: k_eri_f<Eri2011f><<<blocks, threads, 0, s>>>(pr, bt, tasks, ntask, store); break;
      case 9: k_eri_f<Eri2020f><<<blocks, threads, 0, s>>>(pr, bt, tasks, ntask, store); break;
      case 10: k_eri_f<Eri2100f><<<blocks, threads, 0, s>>>(pr, bt, tasks, ntask, store); break;
      case 11: k_eri_f<Eri2110f><<<blocks, threads, 0, s>>>(pr, bt, tasks, ntask, store); break;
      case 12: k_eri_f<Eri2111f><<<blocks, threads, 0, s>>>(pr, bt, tasks, ntask, store); break;
      case 13: k_eri_f<Eri2120f><<<blocks, threads, 0, s>>>(pr, bt, tasks, ntask, store); break;
      default: return PCG_ERR_ARG;
    }
  }
  PCG_CUDA(cudaGetLastError());
  return PCG_OK;
}
