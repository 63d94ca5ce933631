// Internal (non-ABI) declarations shared by the library's translation units.
#pragma once
#include <cuda_runtime.h>

#include "common.cuh"

struct DeviceState {
  double* boys_c = nullptr;
  double* boys_ex = nullptr;
  float* boys_cf = nullptr;
  float* boys_exf = nullptr;
};

DeviceState* pcg_state();
int pcg_ensure_boys(BoysTable* out);

int pcg_launch_pair_data(const DevBasis& b, int npair, const int* pA, const int* pB, const int* ppoff,
                         double* AB, double* zeta, double* P, double* PA, double* K, float* Kf, double* oo2z,
                         cudaStream_t s);
int pcg_launch_one_electron(const DevBasis& b, const BoysTable& bt, int npair, const int* pA, const int* pB,
                            double* S, double* H, cudaStream_t s);

// ERI class table: 21 classes (la lb|lc ld) with la>=lb, lc>=ld, pair class bra >= ket
int pcg_class_id(int la, int lb, int lc, int ld);
int pcg_class_nout(int cls);

// primitive-pair arrays beyond DevPairs (kept separate for the float path)
struct DevPairsExt {
  DevPairs p;
  const double* oo2z;  // 1/(2 zeta) per primitive pair
};

int pcg_launch_eri(int cls, const DevBasis& b, const DevPairsExt& pr, const BoysTable& bt, const int2* tasks,
                   int ntask, double* store, int precision, float fp32_below, const double* qpair,
                   cudaStream_t s);
int pcg_launch_pair_data_f32(int npp, const double* zeta, const double* PA, const double* oo2z, const float* Kf,
                             float* pf8, cudaStream_t s);
int pcg_launch_pair_ao(const DevBasis& b, int npair, const int* pA, const int* pB, int* ao4, cudaStream_t s);
int pcg_launch_digest(int cls, const DevBasis& b, const DevPairsExt& pr, const int2* tasks, int ntask,
                      const double* store, const double* D, double* G, cudaStream_t s);
int pcg_launch_dense(int cls, const DevBasis& b, const DevPairsExt& pr, const int2* tasks, int ntask,
                     const double* store, double* eri, cudaStream_t s);
