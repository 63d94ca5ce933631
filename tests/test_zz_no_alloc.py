"""pcg_fock_build_noalloc against the allocating Fock path.

Some callers of this library cannot allocate GPU memory when they build a Fock
matrix -- their device memory belongs to another allocator or to a pool fixed at
start-up -- so the library offers one entry point whose scratch accumulator is a
static device array.  This test calls it through the C ABI twice in a row, with two
different densities, and checks each result against the ordinary entry points
(pcg_digest_class per class + pcg_fock_build with a caller-allocated accumulator)
within the 1e-10 Fock tolerance used by the other tests; the second call also shows
that the shared array is cleared between calls.  Collected last on purpose.
"""
import ctypes
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _noalloc_fock(eng, D):
    from pychem_gb300 import _lib
    keys = [(cls, part) for cls, rec in sorted(eng.classes.items()) for part in sorted(rec)]
    n = len(keys)
    cls = (ctypes.c_int * n)(*[k[0] for k in keys])
    ntask = (ctypes.c_int * n)(*[eng.classes[c][p][1] for c, p in keys])
    tasks = (ctypes.c_void_p * n)(*[eng.classes[c][p][0].data_ptr() for c, p in keys])
    stores = (ctypes.c_void_p * n)(*[eng.stores[k].data_ptr() for k in keys])
    F = torch.empty(eng.nbf, eng.nbf, dtype=torch.float64, device=D.device)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.call("pcg_fock_build_noalloc", ctypes.byref(eng.basis_t), ctypes.byref(eng.pairs_t), n,
              ctypes.cast(cls, ctypes.c_void_p), ctypes.cast(tasks, ctypes.c_void_p),
              ctypes.cast(ntask, ctypes.c_void_p), ctypes.cast(stores, ctypes.c_void_p),
              ctypes.c_void_p(eng.H.data_ptr()), ctypes.c_void_p(D.data_ptr()), ctypes.c_void_p(F.data_ptr()), stream)
    torch.cuda.synchronize()
    return F


def test_noalloc_fock_matches_allocating_path(golden_dir):
    from pychem_gb300.engine import GpuEngine
    from pychem_gb300.molecule import Molecule
    g = np.load(os.path.join(golden_dir, "water_dimer_631g.npz"))
    coords = [[str(s), float(z)] + list(map(float, xyz)) for s, z, xyz in zip(g["atoms"], g["charges"], g["coords_bohr"])]
    eng = GpuEngine(Molecule(coords, "6-31G", units="BOHR")).prepare()
    rng = np.random.default_rng(11)
    for call in range(2):
        M = rng.normal(size=(eng.nbf, eng.nbf))
        D = torch.tensor(M @ M.T / eng.nbf, device="cuda")
        ref = eng.fock(D).cpu().numpy()
        got = _noalloc_fock(eng, D).cpu().numpy()
        np.testing.assert_allclose(got, ref, rtol=0, atol=1e-10, err_msg="call %d" % call)


def test_noalloc_fock_near_the_size_limit():
    """21 waters in cc-pVDZ: 504 basis functions, s/p/d shells, close to the 512 limit
    of the static accumulator, so nearly the whole array is cleared and indexed."""
    from pychem_gb300 import workloads as W
    from pychem_gb300.engine import GpuEngine
    from pychem_gb300.molecule import Molecule
    mol = Molecule(W.water_cluster(7, 3, 1, seed=5), "cc-pVDZ")
    assert 480 <= mol.NOrbitals <= 512
    from pychem_gb300.guess import sad_density
    eng = GpuEngine(mol).prepare()
    rng = np.random.default_rng(12)
    D0 = sad_density(mol, device="cuda")
    for call in range(2):
        # a physical (SAD) density, then the same with a small symmetric perturbation
        M = rng.normal(size=(eng.nbf, eng.nbf)) * 1e-3 * call
        D = D0 + torch.tensor(M + M.T, device="cuda")
        ref = eng.fock(D).cpu().numpy()
        got = _noalloc_fock(eng, D).cpu().numpy()
        np.testing.assert_allclose(got, ref, rtol=0, atol=1e-10, err_msg="call %d" % call)


def test_noalloc_rejects_too_many_basis_functions():
    from pychem_gb300 import _lib
    from pychem_gb300._lib import BasisT, PairsT
    b = BasisT()
    b.nbf = 513
    p = PairsT()
    dummy = torch.zeros(1, dtype=torch.float64, device="cuda")
    ptr = ctypes.c_void_p(dummy.data_ptr())
    rc = _lib.load().pcg_fock_build_noalloc(ctypes.byref(b), ctypes.byref(p), 0, None, None, None, None, ptr, ptr, ptr,
                                           ctypes.c_void_p(0))
    assert rc == 5  # PCG_ERR_CAPACITY
    assert b"exceeds the static scratch limit" in _lib.load().pcg_last_error()
