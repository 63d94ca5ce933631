// ERI classes 14..17 (see eri_kernels.cuh); split for parallel compilation.
#include "eri_kernels.cuh"

int pcg_launch_eri_g2(int cls, const DevPairsExt& pr, const BoysTable& bt, const int2* tasks, int ntask,
                      double* store, int precision, cudaStream_t s) {
  const int threads = 128, blocks = (ntask + threads - 1) / threads;
  if (precision == 0) {
    switch (cls) {
      case 14: k_eri<Eri2121><<<blocks, threads, 0, s>>>(pr, bt, tasks, ntask, store); break;
      case 15: k_eri<Eri2200><<<blocks, threads, 0, s>>>(pr, bt, tasks, ntask, store); break;
      case 16: k_eri<Eri2210><<<blocks, threads, 0, s>>>(pr, bt, tasks, ntask, store); break;
      case 17: k_eri<Eri2211><<<blocks, threads, 0, s>>>(pr, bt, tasks, ntask, store); break;
      default: return PCG_ERR_ARG;
    }
  } else {
    switch (cls) {
      case 14: k_eri_f<Eri2121f><<<blocks, threads, 0, s>>>(pr, bt, tasks, ntask, store); break;
      case 15: k_eri_f<Eri2200f><<<blocks, threads, 0, s>>>(pr, bt, tasks, ntask, store); break;
      case 16: k_eri_f<Eri2210f><<<blocks, threads, 0, s>>>(pr, bt, tasks, ntask, store); break;
      case 17: k_eri_f<Eri2211f><<<blocks, threads, 0, s>>>(pr, bt, tasks, ntask, store); break;
      default: return PCG_ERR_ARG;
    }
  }
  PCG_CUDA(cudaGetLastError());
  return PCG_OK;
}
