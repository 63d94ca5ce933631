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
int pcg_launch_eri_s0(int cls, const DevPairsExt& pr, const int2* tasks, int ntask, double S, double* store,
                      cudaStream_t s);
int pcg_launch_eri_s1(int cls, const DevPairsExt& pr, const int2* tasks, int ntask, double S, double* store,
                      cudaStream_t s);
int pcg_launch_eri_s2(int cls, const DevPairsExt& pr, const int2* tasks, int ntask, double S, double* store,
                      cudaStream_t s);
int pcg_launch_eri_s3(int cls, const DevPairsExt& pr, const int2* tasks, int ntask, double S, double* store,
                      cudaStream_t s);
int pcg_launch_scattering(int cls, const DevPairsExt& pr, const int2* tasks, int ntask, double S, double* store,
                          cudaStream_t s);
int pcg_launch_digest(int cls, const DevBasis& b, const DevPairsExt& pr, const int2* tasks, int ntask,
                      const double* store, const double* D, double* G, cudaStream_t s);
int pcg_launch_digest_u(int cls, const DevBasis& b, const DevPairsExt& pr, const int2* tasks, int ntask,
                        const double* store, const double* Da, const double* Db, double* GJ, double* GKa,
                        double* GKb, cudaStream_t s);
int pcg_launch_digest_co(int cls, const DevBasis& b, const DevPairsExt& pr, const int2* tasks, int ntask,
                         const double* store, int nd, const double* W, double* GJ, double* GK, cudaStream_t s);
int pcg_launch_dense_pairs(int cls, const DevBasis& b, const DevPairsExt& pr, const int2* tasks, int ntask,
                           const double* store, const int* pmap, double* E, cudaStream_t s);
int pcg_launch_sym_pairs(int cls, const DevBasis& b, const DevPairsExt& pr, const int2* tasks, int ntask,
                         const double* store, const int* pmap, long long rows, double* M, cudaStream_t s);
int pcg_launch_mark_pairs(const int2* tasks, int ntask, unsigned char* used, cudaStream_t s);
int pcg_launch_pair_colmap(int n, const int* pmap, int* colmap, cudaStream_t s);
int pcg_launch_unpack_rows(long long R, int n, int len, const int* colmap, const double* in, double* out,
                           cudaStream_t s);
int pcg_launch_dense(int cls, const DevBasis& b, const DevPairsExt& pr, const int2* tasks, int ntask,
                     const double* store, double* eri, cudaStream_t s);

// Quartet block shapes (2la+1, 2lb+1, 2lc+1, 2ld+1) of the 21 ERI classes, for the
// per-class kernel switches.
#define PCG_SHAPE_CASES(X)                                                                               \
  X(0, 1, 1, 1, 1) X(1, 3, 1, 1, 1) X(2, 3, 1, 3, 1) X(3, 3, 3, 1, 1) X(4, 3, 3, 3, 1) X(5, 3, 3, 3, 3) \
  X(6, 5, 1, 1, 1) X(7, 5, 1, 3, 1) X(8, 5, 1, 3, 3) X(9, 5, 1, 5, 1) X(10, 5, 3, 1, 1)                 \
  X(11, 5, 3, 3, 1) X(12, 5, 3, 3, 3) X(13, 5, 3, 5, 1) X(14, 5, 3, 5, 3) X(15, 5, 5, 1, 1)             \
  X(16, 5, 5, 3, 1) X(17, 5, 5, 3, 3) X(18, 5, 5, 5, 1) X(19, 5, 5, 5, 3) X(20, 5, 5, 5, 5)
