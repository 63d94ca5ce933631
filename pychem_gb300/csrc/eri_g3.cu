// ERI classes 18..19 (see eri_kernels.cuh); split for parallel compilation.
#include "eri_kernels.cuh"

int pcg_launch_eri_g3(int cls, const DevPairsExt& pr, const BoysTable& bt, const int2* tasks, int ntask,
                      double* store, int precision, cudaStream_t s) {
  const int threads = 128, blocks = (ntask + threads - 1) / threads;
  if (precision == 0) {
    switch (cls) {
      case 18: k_eri<Eri2220><<<blocks, threads, 0, s>>>(pr, bt, tasks, ntask, store); break;
      case 19: k_eri<Eri2221><<<blocks, threads, 0, s>>>(pr, bt, tasks, ntask, store); break;
      default: return PCG_ERR_ARG;
    }
  } else {
    switch (cls) {
      case 18: k_eri_f<Eri2220f><<<blocks, threads, 0, s>>>(pr, bt, tasks, ntask, store); break;
      case 19: k_eri_f<Eri2221f><<<blocks, threads, 0, s>>>(pr, bt, tasks, ntask, store); break;
      default: return PCG_ERR_ARG;
    }
  }
  PCG_CUDA(cudaGetLastError());
  return PCG_OK;
}
