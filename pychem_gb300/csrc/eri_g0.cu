// ERI classes 0..5 (see eri_kernels.cuh); split for parallel compilation.
#include "eri_kernels.cuh"

int pcg_launch_eri_g0(int cls, const DevPairsExt& pr, const BoysTable& bt, const int2* tasks, int ntask,
                      double* store, int precision, cudaStream_t s) {
  const int threads = 128, blocks = (ntask + threads - 1) / threads;
  if (precision == 0) {
    switch (cls) {
      case 0: k_eri<Eri0000><<<blocks, threads, 0, s>>>(pr, bt, tasks, ntask, store); break;
      case 1: k_eri<Eri1000><<<blocks, threads, 0, s>>>(pr, bt, tasks, ntask, store); break;
      case 2: k_eri<Eri1010><<<blocks, threads, 0, s>>>(pr, bt, tasks, ntask, store); break;
      case 3: k_eri<Eri1100><<<blocks, threads, 0, s>>>(pr, bt, tasks, ntask, store); break;
      case 4: k_eri<Eri1110><<<blocks, threads, 0, s>>>(pr, bt, tasks, ntask, store); break;
      case 5: k_eri<Eri1111><<<blocks, threads, 0, s>>>(pr, bt, tasks, ntask, store); break;
      default: return PCG_ERR_ARG;
    }
  } else {
    switch (cls) {
      case 0: k_eri_f<Eri0000f><<<blocks, threads, 0, s>>>(pr, bt, tasks, ntask, store); break;
      case 1: k_eri_f<Eri1000f><<<blocks, threads, 0, s>>>(pr, bt, tasks, ntask, store); break;
      case 2: k_eri_f<Eri1010f><<<blocks, threads, 0, s>>>(pr, bt, tasks, ntask, store); break;
      case 3: k_eri_f<Eri1100f><<<blocks, threads, 0, s>>>(pr, bt, tasks, ntask, store); break;
      case 4: k_eri_f<Eri1110f><<<blocks, threads, 0, s>>>(pr, bt, tasks, ntask, store); break;
      case 5: k_eri_f<Eri1111f><<<blocks, threads, 0, s>>>(pr, bt, tasks, ntask, store); break;
      default: return PCG_ERR_ARG;
    }
  }
  PCG_CUDA(cudaGetLastError());
  return PCG_OK;
}
