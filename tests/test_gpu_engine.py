"""GPU integrals, RHF and MP2 against the upstream reference's golden outputs.

Tolerances (from the task's parity bar): S, H and ERIs within 1e-10; total RHF and
MP2 energies within 1e-8 Eh.
"""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

CASES = ["h2o_sto3g", "h2o_631g", "h2o_ccpvdz", "water_dimer_631g"]


def golden(golden_dir, name):
    return np.load(os.path.join(golden_dir, name + ".npz"))


def molecule_of(g):
    from pychem_gb300.molecule import Molecule
    coords = [[str(s), float(z)] + list(map(float, xyz)) for s, z, xyz in zip(g["atoms"], g["charges"], g["coords_bohr"])]
    return Molecule(coords, str(g["basis"]), units="BOHR")


def unpack8(packed, n):
    from oracle.oracle import unpack8 as u
    return u(packed, n)


@pytest.fixture(scope="module")
def engines(golden_dir):
    from pychem_gb300.engine import GpuEngine
    out = {}
    for name in CASES:
        g = golden(golden_dir, name)
        out[name] = (g, GpuEngine(molecule_of(g)).prepare())
    return out


@pytest.mark.parametrize("name", CASES)
def test_one_electron_matrices(engines, name):
    g, eng = engines[name]
    np.testing.assert_allclose(eng.S.cpu().numpy(), g["S"], rtol=0, atol=1e-10)
    np.testing.assert_allclose(eng.H.cpu().numpy(), g["H"], rtol=0, atol=1e-10)


@pytest.mark.parametrize("name", CASES)
def test_eri_tensor(engines, name):
    g, eng = engines[name]
    n = eng.nbf
    ref = g["eri_dense"] if "eri_dense" in g else unpack8(g["eri_packed"], n)
    got = eng.dense_eri().cpu().numpy()
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-10)


@pytest.mark.parametrize("name", CASES)
def test_rhf_energy(engines, name):
    from pychem_gb300.scf import rhf
    g, eng = engines[name]
    r = rhf(eng)
    assert r.converged
    if name == "water_dimer_631g":
        # upstream's DIIS diverges here (its loop prints -163.95); the variational
        # minimum from the oracle's consistent SCF on the same integrals:
        assert abs(r.E - (-151.952697542515)) < 1e-8
    else:
        assert abs(r.E - float(g["E_rhf"])) < 1e-8


@pytest.mark.parametrize("name", ["h2o_631g", "water_dimer_631g"])
def test_core_and_sad_guess_agree(engines, name):
    from pychem_gb300.scf import rhf
    g, eng = engines[name]
    a, b = rhf(eng, guess="core"), rhf(eng, guess="sad")
    assert a.converged and b.converged
    assert abs(a.E - b.E) < 1e-9


@pytest.mark.parametrize("name", ["h2o_sto3g", "h2o_631g"])
def test_mp2_energy(engines, name):
    from pychem_gb300.scf import rhf, rmp2
    g, eng = engines[name]
    r = rhf(eng)
    e2 = rmp2(eng, r.C, r.eps)
    assert abs(e2 - float(g["E_mp2_corr"])) < 1e-8
    assert abs(r.E + e2 - float(g["E_mp2_total"])) < 1e-8


def test_fock_matches_dense_contraction(engines):
    """Digestion of the in-core store equals einsum over the dense tensor
    (upstream hartree_fock.py:345-355) for a random symmetric density."""
    g, eng = engines["water_dimer_631g"]
    n = eng.nbf
    rng = np.random.default_rng(5)
    M = rng.normal(size=(n, n))
    D = torch.tensor(M @ M.T / n, device="cuda")
    F = eng.fock(D).cpu().numpy()
    eri = eng.dense_eri().cpu().numpy()
    Dn = D.cpu().numpy()
    J = np.einsum("cd,abcd->ab", 2 * Dn, eri)
    K = np.einsum("cb,abcd->ad", Dn, eri)
    np.testing.assert_allclose(F, eng.H.cpu().numpy() + J - K, rtol=0, atol=1e-10)


def test_mixed_precision_energy_error(engines):
    from pychem_gb300.engine import GpuEngine
    from pychem_gb300.scf import rhf
    g, eng = engines["water_dimer_631g"]
    mixed = GpuEngine(eng.mol, precision="mixed", fp32_below=1e-4).prepare()
    assert mixed.stats["quartets_fp32"] > 0
    assert mixed.stats["quartets"] == eng.stats["quartets"]
    e64 = rhf(eng).E
    e32 = rhf(mixed).E
    assert abs(e32 - e64) < 1e-8, e32 - e64
