// Electron-scattering integral classes 0..13 (see eri_scat.cuh); split for parallel compilation.
#include "eri_scat.cuh"

int pcg_launch_eri_s0(int cls, const DevPairsExt& pr, const int2* tasks, int ntask, double S, double* store,
                      cudaStream_t s) {
  const int threads = 128, blocks = (ntask + threads - 1) / threads;
  switch (cls) {
      case 0: k_eri_s<Eri0000><<<blocks, threads, 0, s>>>(pr, tasks, ntask, S, store); break;
      case 1: k_eri_s<Eri1000><<<blocks, threads, 0, s>>>(pr, tasks, ntask, S, store); break;
      case 2: k_eri_s<Eri1010><<<blocks, threads, 0, s>>>(pr, tasks, ntask, S, store); break;
      case 3: k_eri_s<Eri1100><<<blocks, threads, 0, s>>>(pr, tasks, ntask, S, store); break;
      case 4: k_eri_s<Eri1110><<<blocks, threads, 0, s>>>(pr, tasks, ntask, S, store); break;
      case 5: k_eri_s<Eri1111><<<blocks, threads, 0, s>>>(pr, tasks, ntask, S, store); break;
      case 6: k_eri_s<Eri2000><<<blocks, threads, 0, s>>>(pr, tasks, ntask, S, store); break;
      case 7: k_eri_s<Eri2010><<<blocks, threads, 0, s>>>(pr, tasks, ntask, S, store); break;
      case 8: k_eri_s<Eri2011><<<blocks, threads, 0, s>>>(pr, tasks, ntask, S, store); break;
      case 9: k_eri_s<Eri2020><<<blocks, threads, 0, s>>>(pr, tasks, ntask, S, store); break;
      case 10: k_eri_s<Eri2100><<<blocks, threads, 0, s>>>(pr, tasks, ntask, S, store); break;
      case 11: k_eri_s<Eri2110><<<blocks, threads, 0, s>>>(pr, tasks, ntask, S, store); break;
      case 12: k_eri_s<Eri2111><<<blocks, threads, 0, s>>>(pr, tasks, ntask, S, store); break;
      case 13: k_eri_s<Eri2120><<<blocks, threads, 0, s>>>(pr, tasks, ntask, S, store); break;
    default: return PCG_ERR_ARG;
  }
  PCG_CUDA(cudaGetLastError());
  return PCG_OK;
}
