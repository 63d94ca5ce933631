"""UHF / CUHF / UMP2 on the GPU against fixtures generated from the upstream reference
(tests/golden/make_golden_open_shell.py) and against the CPU oracle."""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = ["h3_cuhf_sto3g", "h3_uhf_631g", "oh_uhf_631g", "oh_cuhf_631g", "h2o_cation_uhf_631g"]


def _engine(g):
    from pychem_gb300.engine import GpuEngine
    from pychem_gb300.molecule import Molecule
    coords = [[str(a), float(z), *map(float, xyz)] for a, z, xyz in zip(g["atoms"], g["charges"], g["coords_bohr"])]
    mol = Molecule(coords, str(g["basis"]), charge=int(g["charge"]), multiplicity=int(g["multiplicity"]),
                   units="BOHR")
    return GpuEngine(mol).prepare()


@pytest.mark.parametrize("name", CASES)
def test_energies_against_reference(name):
    from pychem_gb300.scf import uhf, ump2
    g = np.load(os.path.join(HERE, "golden", name + ".npz"))
    eng = _engine(g)
    assert np.abs(eng.S.cpu().numpy() - g["S"]).max() < 1e-10
    r = uhf(eng, cuhf=str(g["reference"]) == "CUHF")
    assert r.converged
    assert abs(r.E - float(g["E_scf"])) < 1e-8
    if "E_mp2_corr" in g:
        for gemm in ("ozaki", "fp64"):
            assert abs(ump2(eng, r, gemm=gemm) - float(g["E_mp2_corr"])) < 1e-8


def test_unrestricted_fock_against_oracle():
    from oracle import oracle as O
    g = np.load(os.path.join(HERE, "golden", "oh_uhf_631g.npz"))
    eng = _engine(g)
    n = eng.nbf
    rng = np.random.default_rng(3)
    Da = rng.normal(size=(n, n)); Da = 0.1 * (Da + Da.T)
    Db = rng.normal(size=(n, n)); Db = 0.1 * (Db + Db.T)
    Fa, Fb = eng.fock_u(torch.as_tensor(Da, device="cuda"), torch.as_tensor(Db, device="cuda"))
    eri = g["eri_dense"]
    J = np.einsum("cd,abcd->ab", Da + Db, eri)
    Ka = np.einsum("cb,abcd->ad", Da, eri)
    Kb = np.einsum("cb,abcd->ad", Db, eri)
    assert np.abs(Fa.cpu().numpy() - (g["H"] + J - Ka)).max() < 1e-10
    assert np.abs(Fb.cpu().numpy() - (g["H"] + J - Kb)).max() < 1e-10
    # equal spin densities reproduce the closed-shell Fock build
    Fr = eng.fock(torch.as_tensor(Da, device="cuda")).cpu().numpy()
    Fa2, Fb2 = eng.fock_u(torch.as_tensor(Da, device="cuda"), torch.as_tensor(Da, device="cuda"))
    assert np.abs(Fa2.cpu().numpy() - Fr).max() < 1e-12 and np.abs(Fb2.cpu().numpy() - Fr).max() < 1e-12
