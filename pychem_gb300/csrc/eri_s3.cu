// Electron-scattering integral classes 20 (see eri_scat.cuh); split for parallel compilation.
#include "eri_scat.cuh"

int pcg_launch_eri_s3(int cls, const DevPairsExt& pr, const int2* tasks, int ntask, double S, double* store,
                      cudaStream_t s) {
  const int threads = 128, blocks = (ntask + threads - 1) / threads;
  switch (cls) {
      case 20: k_eri_s<Eri2222><<<blocks, threads, 0, s>>>(pr, tasks, ntask, S, store); break;
    default: return PCG_ERR_ARG;
  }
  PCG_CUDA(cudaGetLastError());
  return PCG_OK;
}
