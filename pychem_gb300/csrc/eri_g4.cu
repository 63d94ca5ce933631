// ERI class 20, (dd|dd), double precision (see eri_kernels.cuh); its own translation
// unit because it is the largest straight-line kernel.
#include "eri_kernels.cuh"

int pcg_launch_eri_g4(int cls, const DevPairsExt& pr, const BoysTable& bt, const int2* tasks, int ntask,
                      double* store, int precision, cudaStream_t s) {
  const int threads = 128, blocks = (ntask + threads - 1) / threads;
  if (cls != 20 || precision != 0) return PCG_ERR_ARG;
  k_eri<Eri2222><<<blocks, threads, 0, s>>>(pr, bt, tasks, ntask, store);
  PCG_CUDA(cudaGetLastError());
  return PCG_OK;
}
