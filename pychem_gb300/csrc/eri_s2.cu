// Electron-scattering integral classes 18..19 (see eri_scat.cuh); split for parallel compilation.
#include "eri_scat.cuh"

int pcg_launch_eri_s2(int cls, const DevPairsExt& pr, const int2* tasks, int ntask, double S, double* store,
                      cudaStream_t s) {
  const int threads = 128, blocks = (ntask + threads - 1) / threads;
  switch (cls) {
      case 18: k_eri_s<Eri2220><<<blocks, threads, 0, s>>>(pr, tasks, ntask, S, store); break;
      case 19: k_eri_s<Eri2221><<<blocks, threads, 0, s>>>(pr, tasks, ntask, S, store); break;
    default: return PCG_ERR_ARG;
  }
  PCG_CUDA(cudaGetLastError());
  return PCG_OK;
}
