// C ABI of the batched layer (include/pychem_gb300.h, section 2) and error handling.
#include <stdio.h>
#include <string.h>

#include "../../include/pychem_gb300.h"
#include "common.cuh"
#include "pcg_internal.h"

static thread_local char g_err[512] = "";

void pcg_set_error(const char* msg) { snprintf(g_err, sizeof(g_err), "%s", msg); }
void pcg_set_cuda_error(cudaError_t e, const char* what) {
  snprintf(g_err, sizeof(g_err), "CUDA error %d (%s) in %s", (int)e, cudaGetErrorString(e), what);
}

int pcg_launch_schwarz(int cls, const int2* tasks, int ntask, const double* store, double* Q, cudaStream_t s);
int pcg_launch_expand(int nbra, const int* bra, const int* ket, const long long* off, const int* qstart,
                      const int* diag, long long ntask, int2* out, cudaStream_t s);
int pcg_launch_fock(int n, const double* H, const double* G, double* F, cudaStream_t s);
int pcg_launch_fock_batched(int nblocks, int ld, const double* H, const double* G, double* F, cudaStream_t s);

static DevBasis to_dev(const pcg_basis_t* b) {
  DevBasis d;
  d.nshell = b->nshell; d.nprim = b->nprim; d.natom = b->natom; d.nbf = b->nbf;
  d.sh_l = b->sh_l; d.sh_nprim = b->sh_nprim; d.sh_prim = b->sh_prim; d.sh_ao = b->sh_ao;
  d.sh_atom = b->sh_atom; d.sh_xyz = b->sh_xyz; d.pr_exp = b->pr_exp; d.pr_cc = b->pr_cc;
  d.at_xyz = b->at_xyz; d.at_z = b->at_z;
  d.ld = b->ld > 0 ? b->ld : b->nbf;
  d.sh_blk = b->sh_blk; d.sh_at0 = b->sh_at0; d.sh_nat = b->sh_nat;
  return d;
}

static DevPairsExt to_dev(const pcg_pairs_t* p) {
  DevPairsExt d;
  d.p.npair = p->npair; d.p.npp = p->npp;
  d.p.A = p->A; d.p.B = p->B; d.p.ppoff = p->ppoff; d.p.npp_of = p->npp_of;
  d.p.AB = p->AB; d.p.zeta = p->zeta; d.p.P = p->P; d.p.PA = p->PA; d.p.K = p->K; d.p.Kf = p->Kf;
  d.p.ao4 = (const int4*)p->ao4;
  d.p.pf8 = (const float4*)p->pf8;
  d.oo2z = p->oo2z;
  return d;
}

extern "C" {

int pcg_version(void) { return 1; }

const char* pcg_last_error(void) { return g_err; }

int pcg_device_init(void) {
  BoysTable bt;
  return pcg_ensure_boys(&bt);
}

int pcg_pair_data(const pcg_basis_t* basis, int npair, const int* A, const int* B, const int* ppoff,
                  double* AB, double* zeta, double* P, double* PA, double* K, float* Kf, double* oo2z,
                  void* stream) {
  if (!basis || npair < 0) { pcg_set_error("pcg_pair_data: bad arguments"); return PCG_ERR_ARG; }
  return pcg_launch_pair_data(to_dev(basis), npair, A, B, ppoff, AB, zeta, P, PA, K, Kf, oo2z,
                              (cudaStream_t)stream);
}

int pcg_pair_data_f32(int npp, const double* zeta, const double* PA, const double* oo2z, const float* Kf, float* pf8,
                      void* stream) {
  if (npp < 0 || (npp > 0 && (!zeta || !PA || !oo2z || !Kf || !pf8))) {
    pcg_set_error("pcg_pair_data_f32: bad arguments");
    return PCG_ERR_ARG;
  }
  return pcg_launch_pair_data_f32(npp, zeta, PA, oo2z, Kf, pf8, (cudaStream_t)stream);
}

int pcg_pair_ao(const pcg_basis_t* basis, int npair, const int* A, const int* B, int* ao4, void* stream) {
  if (!basis || npair < 0 || (npair > 0 && (!A || !B || !ao4))) {
    pcg_set_error("pcg_pair_ao: bad arguments");
    return PCG_ERR_ARG;
  }
  return pcg_launch_pair_ao(to_dev(basis), npair, A, B, ao4, (cudaStream_t)stream);
}

int pcg_one_electron(const pcg_basis_t* basis, int npair, const int* A, const int* B, double* S, double* H,
                     void* stream) {
  if (!basis || npair < 0) { pcg_set_error("pcg_one_electron: bad arguments"); return PCG_ERR_ARG; }
  BoysTable bt;
  int rc = pcg_ensure_boys(&bt);
  if (rc) return rc;
  return pcg_launch_one_electron(to_dev(basis), bt, npair, A, B, S, H, (cudaStream_t)stream);
}

int pcg_eri_class_id(int la, int lb, int lc, int ld) { return pcg_class_id(la, lb, lc, ld); }

int pcg_eri_class_nout(int cls) { return pcg_class_nout(cls); }

int pcg_eri_class(int cls, const pcg_basis_t* basis, const pcg_pairs_t* pairs, const int* tasks, int ntask,
                  double* store, int fp32, void* stream) {
  if (cls < 0 || cls > 20 || !basis || !pairs || ntask < 0) {
    pcg_set_error("pcg_eri_class: bad arguments");
    return PCG_ERR_ARG;
  }
  BoysTable bt;
  int rc = pcg_ensure_boys(&bt);
  if (rc) return rc;
  return pcg_launch_eri(cls, to_dev(basis), to_dev(pairs), bt, (const int2*)tasks, ntask, store, fp32 ? 1 : 0,
                        0.0f, nullptr, (cudaStream_t)stream);
}

int pcg_schwarz_class(int cls, const int* tasks, int ntask, const double* store, double* Q, void* stream) {
  int rc = pcg_launch_schwarz(cls, (const int2*)tasks, ntask, store, Q, (cudaStream_t)stream);
  if (rc == PCG_ERR_ARG) pcg_set_error("pcg_schwarz_class: not a diagonal class");
  return rc;
}

int pcg_expand_tasks(int nbra, const int* bra, const int* ket, const long long* off, const int* qstart,
                     const int* diag, long long ntask, int* out_tasks, void* stream) {
  if (nbra <= 0 && ntask > 0) { pcg_set_error("pcg_expand_tasks: no bra pairs"); return PCG_ERR_ARG; }
  return pcg_launch_expand(nbra, bra, ket, off, qstart, diag, ntask, (int2*)out_tasks, (cudaStream_t)stream);
}

int pcg_digest_class(int cls, const pcg_basis_t* basis, const pcg_pairs_t* pairs, const int* tasks, int ntask,
                     const double* store, const double* D, double* G, void* stream) {
  if (cls < 0 || cls > 20 || !basis || !pairs) { pcg_set_error("pcg_digest_class: bad arguments"); return PCG_ERR_ARG; }
  return pcg_launch_digest(cls, to_dev(basis), to_dev(pairs), (const int2*)tasks, ntask, store, D, G,
                           (cudaStream_t)stream);
}

int pcg_digest_class_u(int cls, const pcg_basis_t* basis, const pcg_pairs_t* pairs, const int* tasks, int ntask,
                       const double* store, const double* Da, const double* Db, double* GJ, double* GKa, double* GKb,
                       void* stream) {
  if (cls < 0 || cls > 20 || !basis || !pairs || !Da || !Db || !GJ || !GKa || !GKb) {
    pcg_set_error("pcg_digest_class_u: bad arguments");
    return PCG_ERR_ARG;
  }
  return pcg_launch_digest_u(cls, to_dev(basis), to_dev(pairs), (const int2*)tasks, ntask, store, Da, Db, GJ, GKa,
                             GKb, (cudaStream_t)stream);
}

int pcg_scattering_class(int cls, const pcg_basis_t* basis, const pcg_pairs_t* pairs, const int* tasks, int ntask,
                         double S, double* store, void* stream) {
  if (cls < 0 || cls > 20 || !basis || !pairs || ntask < 0 || !(S >= 0.0)) {
    pcg_set_error("pcg_scattering_class: bad arguments");
    return PCG_ERR_ARG;
  }
  return pcg_launch_scattering(cls, to_dev(pairs), (const int2*)tasks, ntask, S, store, (cudaStream_t)stream);
}

int pcg_digest_class_co(int cls, const pcg_basis_t* basis, const pcg_pairs_t* pairs, const int* tasks, int ntask,
                        const double* store, int nd, const double* W, double* GJ, double* GK, void* stream) {
  if (cls < 0 || cls > 20 || !basis || !pairs || nd < 0 || (nd > 0 && (!W || !GJ || !GK))) {
    pcg_set_error("pcg_digest_class_co: bad arguments");
    return PCG_ERR_ARG;
  }
  if (basis->sh_blk) { pcg_set_error("pcg_digest_class_co: one molecule only"); return PCG_ERR_UNSUPPORTED; }
  return pcg_launch_digest_co(cls, to_dev(basis), to_dev(pairs), (const int2*)tasks, ntask, store, nd, W, GJ, GK,
                              (cudaStream_t)stream);
}

int pcg_fock_build(int n, const double* H, const double* G, double* F, void* stream) {
  return pcg_launch_fock(n, H, G, F, (cudaStream_t)stream);
}

int pcg_fock_build_batched(int nblocks, int ld, const double* H, const double* G, double* F, void* stream) {
  if (nblocks < 1 || ld < 1) { pcg_set_error("pcg_fock_build_batched: bad arguments"); return PCG_ERR_ARG; }
  return pcg_launch_fock_batched(nblocks, ld, H, G, F, (cudaStream_t)stream);
}

int pcg_dense_class(int cls, const pcg_basis_t* basis, const pcg_pairs_t* pairs, const int* tasks, int ntask,
                    const double* store, double* eri, void* stream) {
  if (cls < 0 || cls > 20 || !basis || !pairs) { pcg_set_error("pcg_dense_class: bad arguments"); return PCG_ERR_ARG; }
  if (basis->sh_blk) { pcg_set_error("pcg_dense_class: one molecule only"); return PCG_ERR_UNSUPPORTED; }
  return pcg_launch_dense(cls, to_dev(basis), to_dev(pairs), (const int2*)tasks, ntask, store, eri,
                          (cudaStream_t)stream);
}

int pcg_dense_pairs_class(int cls, const pcg_basis_t* basis, const pcg_pairs_t* pairs, const int* tasks, int ntask,
                          const double* store, const int* pairmap, double* E, void* stream) {
  if (cls < 0 || cls > 20 || !basis || !pairs || !E) {
    pcg_set_error("pcg_dense_pairs_class: bad arguments");
    return PCG_ERR_ARG;
  }
  if (basis->sh_blk) { pcg_set_error("pcg_dense_pairs_class: one molecule only"); return PCG_ERR_UNSUPPORTED; }
  return pcg_launch_dense_pairs(cls, to_dev(basis), to_dev(pairs), (const int2*)tasks, ntask, store, pairmap, E,
                                (cudaStream_t)stream);
}

int pcg_sym_pairs_class(int cls, const pcg_basis_t* basis, const pcg_pairs_t* pairs, const int* tasks, int ntask,
                        const double* store, const int* pairmap, long long rows, double* M, void* stream) {
  if (cls < 0 || cls > 20 || !basis || !pairs || !pairmap || rows < 1 || !M || (ntask > 0 && (!tasks || !store))) {
    pcg_set_error("pcg_sym_pairs_class: bad arguments");
    return PCG_ERR_ARG;
  }
  if (basis->sh_blk) { pcg_set_error("pcg_sym_pairs_class: one molecule only"); return PCG_ERR_UNSUPPORTED; }
  return pcg_launch_sym_pairs(cls, to_dev(basis), to_dev(pairs), (const int2*)tasks, ntask, store, pairmap, rows, M,
                              (cudaStream_t)stream);
}

int pcg_mark_pairs(const int* tasks, int ntask, unsigned char* used, void* stream) {
  if (ntask < 0 || !used || (ntask > 0 && !tasks)) {
    pcg_set_error("pcg_mark_pairs: bad arguments");
    return PCG_ERR_ARG;
  }
  return pcg_launch_mark_pairs((const int2*)tasks, ntask, used, (cudaStream_t)stream);
}

int pcg_pair_colmap(int n, const int* pairmap, int* colmap, void* stream) {
  if (n < 1 || n > 46340 || !colmap) {
    pcg_set_error("pcg_pair_colmap: bad arguments");
    return PCG_ERR_ARG;
  }
  return pcg_launch_pair_colmap(n, pairmap, colmap, (cudaStream_t)stream);
}

int pcg_unpack_pairs(long long R, int n, int len, const int* colmap, const double* in, double* out, void* stream) {
  if (R < 0 || n < 1 || n > 46340 || len < 1 || !colmap || !in || !out) {
    pcg_set_error("pcg_unpack_pairs: bad arguments");
    return PCG_ERR_ARG;
  }
  return pcg_launch_unpack_rows(R, n, len, colmap, in, out, (cudaStream_t)stream);
}

}  // extern "C"

// ---------------------------------------------------------------------------------
// Arithmetic-throughput probe: each thread runs 8 independent FMA chains for `iters`
// steps (FP64 when fp32 == 0, else FP32); the result is written so the work is kept.
// Used by bench.py to measure the FP64/FP32 pipe peaks that the ERI roofline uses.
// ---------------------------------------------------------------------------------
template <class T>
__global__ void k_fma_probe(int iters, T* out) {
  T a0 = (T)threadIdx.x * (T)1e-3, a1 = a0 + (T)1, a2 = a0 + (T)2, a3 = a0 + (T)3;
  T a4 = a0 + (T)4, a5 = a0 + (T)5, a6 = a0 + (T)6, a7 = a0 + (T)7;
  const T m = (T)0.999999, c = (T)1e-7;
  for (int i = 0; i < iters; ++i) {
    a0 = fma(a0, m, c); a1 = fma(a1, m, c); a2 = fma(a2, m, c); a3 = fma(a3, m, c);
    a4 = fma(a4, m, c); a5 = fma(a5, m, c); a6 = fma(a6, m, c); a7 = fma(a7, m, c);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}

extern "C" int pcg_fma_probe(int blocks, int threads, int iters, int fp32, void* out, void* stream) {
  if (blocks <= 0 || threads <= 0 || threads > 1024 || iters <= 0 || !out) {
    pcg_set_error("pcg_fma_probe: bad arguments");
    return PCG_ERR_ARG;
  }
  if (fp32) k_fma_probe<float><<<blocks, threads, 0, (cudaStream_t)stream>>>(iters, (float*)out);
  else k_fma_probe<double><<<blocks, threads, 0, (cudaStream_t)stream>>>(iters, (double*)out);
  PCG_CUDA(cudaGetLastError());
  return PCG_OK;
}
