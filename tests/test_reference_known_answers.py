"""The reference's own known answers (``Tests/integration_tests.py``) on CPU.

Where the reference tree is present (``PYCHEM_REFERENCE``, as for the fixture
generators), its test inputs are read with pychem_gb300's input reader and run through
the product's host pipeline with the oracle supplying integrals and the UHF:
LiH spin-flip NOCI (states, NOCI energies, a block of alpha orbitals) and H2 CUHF in
6-311G, compared at the five decimals the reference's tests use where the reference
defines the quantity (see test_lih_spin_flip_noci).  Skipped elsewhere
(the GPU machines have no reference tree); nothing of the reference is copied.
"""
import os
import re
import sys

import numpy as np
import pytest
import torch

from oracle import oracle
from pychem_gb300 import cli, noci
from pychem_gb300.molecule import Molecule
from pychem_gb300.scf import SCFResult

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import refrun  # noqa: E402

TESTS = os.path.join(refrun.REFERENCE, "Tests") if refrun.REFERENCE else ""
pytestmark = pytest.mark.skipif(not os.path.isfile(os.path.join(TESTS, "integration_tests.py")),
                                reason="reference tree not present (set PYCHEM_REFERENCE)")


def expectations():
    """{input file name: {"hf": [...], "noci": [...], "alpha": array}} parsed from the
    reference's test module."""
    text = open(os.path.join(TESTS, "integration_tests.py")).read()
    out = {}
    for block in re.split(r"\nclass ", text)[1:]:
        m = re.search(r'infile_name\s*=\s*"Tests/([^"]+)"', block)
        if not m:
            continue
        rec = {}
        for key, fn in (("hf", "HF_energies_test"), ("noci", "NOCI_energies_test")):
            mm = re.search(fn + r"\(\[([^\]]*)\]\)", block)
            if mm:
                rec[key] = [float(x) for x in mm.group(1).split(",")]
        mm = re.search(r"np\.array\(\[(.*?)\]\)\s*\n\s*self\.alpha_orbitals_test", block, re.S)
        if mm:
            rows = re.findall(r"\[([^\[\]]+)\]", mm.group(1))
            rec["alpha"] = np.array([[float(x) for x in r.split(",")] for r in rows])
        out[m.group(1)] = rec
    return out


class CpuEngine:
    """Oracle integrals behind the attributes noci.hf_states and noci_matrix use."""

    def __init__(self, mol):
        self.mol = mol
        b = oracle.Basis([(a[0], a[1], *a[2]) for a in mol.atoms], mol.Basis)
        S, H = b.one_electron()
        self.S, self.H = torch.tensor(S), torch.tensor(H)
        self.eri = b.eri_dense()
        self.e_nuc = b.nuclear_repulsion()
        self.nbf = mol.NOrbitals

    def coulomb_exchange(self, W):
        E = torch.tensor(self.eri)
        return torch.einsum("ncd,abcd->nab", W, E), torch.einsum("ncb,abcd->nad", W, E)


def oracle_uhf(eng, cuhf=False, max_iter=300, e_tol=1e-10, d_tol=1e-8, C0=None, mom=False, occ=None,
               cuhf_spaces=None):
    na, nb = occ
    c0 = None if C0 is None else (C0[0].numpy(), C0[1].numpy())
    r = oracle.uhf(eng.S.numpy(), eng.H.numpy(), eng.eri, na, nb, eng.e_nuc, cuhf=cuhf, max_iter=max_iter,
                   d_tol=d_tol, C0=c0, mom=mom, cuhf_spaces=cuhf_spaces)
    Ca, Cb, ea, eb = r["Ca"], r["Cb"], r["ea"], r["eb"]
    if mom:
        for C, e, n in ((Ca, ea, na), (Cb, eb, nb)):
            idx = np.argsort(e[:n], kind="stable")
            C[:, :n], e[:n] = C[:, :n][:, idx], e[:n][idx]
    return SCFResult(E=r["E"], Ca=torch.tensor(Ca), Cb=torch.tensor(Cb), ea=torch.tensor(ea), eb=torch.tensor(eb),
                     iterations=r["iterations"], converged=r["converged"])


def molecule(opts):
    coords, units = cli._coords(opts)
    return Molecule(coords, opts["BASIS_SETS"][-1], charge=int(opts.get("CHARGE", 0)),
                    multiplicity=int(opts.get("MULTIPLICITY", 1)), units=units)


def test_lih_spin_flip_noci(monkeypatch):
    """The two Hartree-Fock states and the triplet-derived NOCI root to five decimals.
    The lowest and highest NOCI roots and the ground determinant's orbitals depend on
    the MOM ground state, which the reference does not converge within this input's 50
    iterations: run here, the current reference code itself gives -7.96944 and -7.85947
    for those roots (its test expects -7.96826 and -7.85624) and 0.07423 / 0.10577 for
    the second column of the orbital block (expected 0.06856 / 0.09058).  For them only
    the root order, a 1e-2 band and the core orbital's column (1e-3) are checked."""
    exp = expectations()["LiH_SFS_NOCI.test.inp"]
    (name, opts), = cli.read_sections(os.path.join(TESTS, "LiH_SFS_NOCI.test.inp"))
    assert opts["METHOD"] == "NOCI"
    mol = molecule(opts)
    eng = CpuEngine(mol)
    monkeypatch.setattr(noci, "uhf", oracle_uhf)
    exc = opts["EXCITATIONS"]
    states, sf = noci.excited_states(mol.NAlphaElectrons, mol.NBetaElectrons, mol.NOrbitals, exc)
    res = noci.hf_states(eng, states, spin_flip="SF" in exc, reference=opts["REFERENCE"],
                         constrain_excited=bool(opts.get("CONSTRAIN_EXCITED")), max_iter=300)
    da, db = noci.determinants(states, res, sf)
    # the reference's States after the spin-flip rearrangement carry their HF state's energy
    hf_of_det = [res[i].E for i, _, _ in sf]
    np.testing.assert_almost_equal(hf_of_det[:len(exp["hf"])], exp["hf"], decimal=5)
    H, S = noci.noci_matrix(eng, da, db, mol.NAlphaElectrons, mol.NBetaElectrons)
    from scipy.linalg import eigh
    e = eigh(H.numpy(), S.numpy(), eigvals_only=True)
    np.testing.assert_almost_equal(e[1], exp["noci"][1], decimal=5)
    assert np.all(np.abs(e[:3] - exp["noci"]) < 1e-2) and e[0] < e[1] < e[2]
    x = exp["alpha"].shape[0]
    assert np.abs(np.abs(da[0].numpy()[:x, 0]) - np.abs(exp["alpha"][:, 0])).max() < 1e-3


def test_h2_cuhf_6311g():
    exp = expectations()["H2_HF.test.inp"]
    (name, opts), = cli.read_sections(os.path.join(TESTS, "H2_HF.test.inp"))
    mol = molecule(opts)
    eng = CpuEngine(mol)
    r = oracle.uhf(eng.S.numpy(), eng.H.numpy(), eng.eri, mol.NAlphaElectrons, mol.NBetaElectrons, eng.e_nuc,
                   cuhf=opts["REFERENCE"] == "CUHF")
    np.testing.assert_almost_equal([r["E"]], exp["hf"], decimal=5)


def _printed_table(path):
    text = open(path).read()
    i = text.index("Scattering patterns for each electronic state")
    rows = []
    for line in text[i:].splitlines()[1:]:
        nums = re.findall(r"[-+]?\d+\.\d+(?:[eE][-+]?\d+)?", line)
        if len(nums) == 2:
            rows.append([float(x) for x in nums])
        elif rows:
            break
    return np.array(rows)


@pytest.mark.parametrize("example", ["example5", "example7"])
def test_scattering_examples_at_zero_momentum(example):
    """Tests/example5 and example7 (closed-shell RHF, grid [0.0]): the printed I(0)
    against the oracle's intensity from its own SCF densities, to the printed digits.
    The shipped tables of example2 and example6 (S > 0) come from an older reference:
    run here, the current reference prints 9.0, 7.374809, 4.673569, ... for example2
    and 12.091491, 6.898692, 5.202370, ... for example6 (the oracle matches both to
    1e-6), not the shipped 10.0, 8.164531, ... and 12.179709, 6.898709, 5.057529, ...;
    they are not compared."""
    (name, opts), = cli.read_sections(os.path.join(TESTS, example + ".inp"))
    mol = molecule(opts)
    eng = CpuEngine(mol)
    r = oracle.rhf(eng.S.numpy(), eng.H.numpy(), eng.eri, mol.NAlphaElectrons, eng.e_nuc)
    tab = _printed_table(os.path.join(TESTS, example + ".out"))
    b = oracle.Basis([(a[0], a[1], *a[2]) for a in mol.atoms], mol.Basis)
    for S, printed in tab:
        I = oracle.scattering_intensity(r["D"], r["D"], b.eri_dense(scattering=S), mol.NElectrons)
        assert abs(I - printed) < 1e-10


def test_example3_cuhf_energy():
    """Tests/example3 (CUHF, 6-311G): the printed final Hartree-Fock energy against the
    oracle's CUHF, within the 3e-6 that the reference's |dE| < 1e-7 stop leaves."""
    (name, opts), = cli.read_sections(os.path.join(TESTS, "example3.inp"))
    assert opts["REFERENCE"] == "CUHF"
    mol = molecule(opts)
    eng = CpuEngine(mol)
    r = oracle.uhf(eng.S.numpy(), eng.H.numpy(), eng.eri, mol.NAlphaElectrons, mol.NBetaElectrons, eng.e_nuc,
                   cuhf=True)
    printed = re.findall(r"Final HF energy:\s*([-0-9.eE+]+)", open(os.path.join(TESTS, "example3.out")).read())
    assert printed and abs(r["E"] - float(printed[-1])) < 3e-6
