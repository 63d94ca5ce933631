// Closed-shell Fock build that allocates no device memory.
//
// The ordinary path (pcg_digest_class per class + pcg_fock_build) needs a caller-
// allocated nbf x nbf accumulator G.  Some callers cannot allocate device memory at
// the point where they build a Fock matrix: hosts whose GPU memory is owned by
// another allocator (a framework's caching allocator, or one fixed pool reserved at
// start-up) that gives this library no allocation hook, and hosts that forbid any
// allocation after initialisation.  For them the accumulator lives in the file-scope
// array below, sized for nbf <= PCG_NOALLOC_MAX_NBF (512 basis functions, 2 MiB).
// Every GPU that loads this library holds that array until the process exits.
//
// The array is a device symbol: in host code its name is only a stand-in, so the
// host obtains its device address with cudaGetSymbolAddress, with the calling device
// current, on every call (the lookup allocates nothing; repeating it keeps the address
// right after a cudaDeviceReset reloads the module).  The first call on a device may
// load the library's device code there, so it should come before any stream capture.
// Calls share the one array: each call clears the nbf x nbf block it uses, and calls
// that overlap on the GPU (two streams, or two host threads on one device) race on it
// and must be serialised by the caller.
//
// Every argument is checked before the first CUDA call, so a rejected call launches
// nothing and leaves both F and the shared array untouched.
#include <stdio.h>

#include "../../include/pychem_gb300.h"
#include "common.cuh"
#include "pcg_internal.h"

#define PCG_NOALLOC_MAX_NBF 512

static __device__ __align__(256) double g_fock_scratch[PCG_NOALLOC_MAX_NBF * PCG_NOALLOC_MAX_NBF];

int pcg_launch_fock(int n, const double* H, const double* G, double* F, cudaStream_t s);

static DevBasis basis_of(const pcg_basis_t* b) {
  DevBasis d;
  d.nshell = b->nshell; d.nprim = b->nprim; d.natom = b->natom; d.nbf = b->nbf;
  d.sh_l = b->sh_l; d.sh_nprim = b->sh_nprim; d.sh_prim = b->sh_prim; d.sh_ao = b->sh_ao;
  d.sh_atom = b->sh_atom; d.sh_xyz = b->sh_xyz; d.pr_exp = b->pr_exp; d.pr_cc = b->pr_cc;
  d.at_xyz = b->at_xyz; d.at_z = b->at_z;
  d.ld = b->ld > 0 ? b->ld : b->nbf;
  d.sh_blk = b->sh_blk; d.sh_at0 = b->sh_at0; d.sh_nat = b->sh_nat;
  return d;
}

static DevPairsExt pairs_of(const pcg_pairs_t* p) {
  DevPairsExt d;
  d.p.npair = p->npair; d.p.npp = p->npp;
  d.p.A = p->A; d.p.B = p->B; d.p.ppoff = p->ppoff; d.p.npp_of = p->npp_of;
  d.p.AB = p->AB; d.p.zeta = p->zeta; d.p.P = p->P; d.p.PA = p->PA; d.p.K = p->K; d.p.Kf = p->Kf;
  d.p.ao4 = (const int4*)p->ao4;
  d.p.pf8 = (const float4*)p->pf8;
  d.oo2z = p->oo2z;
  return d;
}

extern "C" int pcg_fock_build_noalloc(const pcg_basis_t* basis, const pcg_pairs_t* pairs, int nclass,
                                      const int* cls, const int* const* tasks, const int* ntask,
                                      const double* const* stores, const double* H, const double* D, double* F,
                                      void* stream) {
  if (!basis || !pairs || nclass < 0 || (nclass > 0 && (!cls || !tasks || !ntask || !stores)) || !H || !D || !F) {
    pcg_set_error("pcg_fock_build_noalloc: bad arguments");
    return PCG_ERR_ARG;
  }
  const int n = basis->nbf;
  if (basis->sh_blk) {
    pcg_set_error("pcg_fock_build_noalloc: one molecule only");
    return PCG_ERR_UNSUPPORTED;
  }
  if (n <= 0 || n > PCG_NOALLOC_MAX_NBF) {
    char msg[160];
    snprintf(msg, sizeof(msg), "pcg_fock_build_noalloc: nbf = %d exceeds the static scratch limit of %d basis functions",
             n, PCG_NOALLOC_MAX_NBF);
    pcg_set_error(msg);
    return PCG_ERR_CAPACITY;
  }
  // the accumulator is addressed with row stride nbf: any other matrix layout would
  // index past the cleared block (and, for ld > 512, past the array)
  if (basis->ld > 0 && basis->ld != n) {
    pcg_set_error("pcg_fock_build_noalloc: basis->ld must be 0 or nbf (one molecule, nbf x nbf matrices)");
    return PCG_ERR_ARG;
  }
  for (int k = 0; k < nclass; ++k) {
    if (cls[k] < 0 || cls[k] > 20 || ntask[k] < 0 || (ntask[k] > 0 && (!tasks[k] || !stores[k]))) {
      char msg[120];
      snprintf(msg, sizeof(msg), "pcg_fock_build_noalloc: bad class entry %d", k);
      pcg_set_error(msg);
      return PCG_ERR_ARG;
    }
  }
  int dev = 0;
  PCG_CUDA(cudaGetDevice(&dev));
  double* G = nullptr;
  PCG_CUDA(cudaGetSymbolAddress((void**)&G, g_fock_scratch));
  cudaStream_t s = (cudaStream_t)stream;
  PCG_CUDA(cudaMemsetAsync(G, 0, sizeof(double) * (size_t)n * n, s));
  DevBasis b = basis_of(basis);
  b.ld = n;
  DevPairsExt pr = pairs_of(pairs);
  // the digestion then reads AO offsets from the shell tables, whose block offset is 0
  // without sh_blk, instead of the optional per-pair table with its own offsets
  pr.p.ao4 = nullptr;
  for (int k = 0; k < nclass; ++k) {
    int rc = pcg_launch_digest(cls[k], b, pr, (const int2*)tasks[k], ntask[k], stores[k], D, G, s);
    if (rc) return rc;
  }
  return pcg_launch_fock(n, H, G, F, s);
}
