// Electron-scattering integral classes 14..17 (see eri_scat.cuh); split for parallel compilation.
#include "eri_scat.cuh"

int pcg_launch_eri_s1(int cls, const DevPairsExt& pr, const int2* tasks, int ntask, double S, double* store,
                      cudaStream_t s) {
  const int threads = 128, blocks = (ntask + threads - 1) / threads;
  switch (cls) {
      case 14: k_eri_s<Eri2121><<<blocks, threads, 0, s>>>(pr, tasks, ntask, S, store); break;
      case 15: k_eri_s<Eri2200><<<blocks, threads, 0, s>>>(pr, tasks, ntask, S, store); break;
      case 16: k_eri_s<Eri2210><<<blocks, threads, 0, s>>>(pr, tasks, ntask, S, store); break;
      case 17: k_eri_s<Eri2211><<<blocks, threads, 0, s>>>(pr, tasks, ntask, S, store); break;
    default: return PCG_ERR_ARG;
  }
  PCG_CUDA(cudaGetLastError());
  return PCG_OK;
}
