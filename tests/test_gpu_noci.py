"""NOCI on the GPU against the reference fixtures and the oracle.

* GpuEngine.coulomb_exchange (unrestricted digestion fed (W, W^T)) against dense
  einsums of the reference's ERI tensor for non-symmetric co-densities;
* the CI matrix from the reference's own determinants, with the J/K of every
  co-density from the ERI store;
* the whole calculation -- state SCFs in the reference's order, spin-flip
  determinants, CI matrix, generalised eigenproblem -- against the reference's
  Hartree-Fock and NOCI energies.
"""
import numpy as np
import pytest
import torch

from pychem_gb300 import noci
from pychem_gb300.engine import GpuEngine
from pychem_gb300.molecule import Molecule

from test_noci_host import NAMES, check_ci_matrix, element_tolerance, energies_defined, load

pytestmark = pytest.mark.gpu


def engine_for(z):
    coords = [[str(a), float(c), *map(float, x)] for a, c, x in zip(z["atoms"], z["charges"], z["coords_bohr"])]
    mol = Molecule(coords, str(z["basis"]), units="BOHR")
    return GpuEngine(mol).prepare()


def test_coulomb_exchange_nonsymmetric():
    z = load("noci_lih_sfs_631g")
    eng = engine_for(z)
    n = eng.nbf
    assert np.abs(eng.S.cpu().numpy() - z["S"]).max() < 1e-12
    g = torch.Generator().manual_seed(7)
    W = torch.randn(3, n, n, generator=g, dtype=torch.float64)
    J, K = eng.coulomb_exchange(W.cuda())
    eri = torch.tensor(z["eri_dense"])
    Jr = torch.einsum("ncd,abcd->nab", W, eri)
    Kr = torch.einsum("ncb,abcd->nad", W, eri)
    assert float((J.cpu() - Jr).abs().max()) < 1e-10
    assert float((K.cpu() - Kr).abs().max()) < 1e-10


@pytest.mark.parametrize("name", NAMES)
def test_ci_matrix_from_reference_determinants(name):
    z = load(name)
    eng = engine_for(z)
    dets_a = [torch.tensor(x, device="cuda") for x in z["det_alpha"]]
    dets_b = [torch.tensor(x, device="cuda") for x in z["det_beta"]]
    H, S, pairs = noci.noci_matrix(eng, dets_a, dets_b, int(z["n_alpha"]), int(z["n_beta"]), return_pairs=True)
    check_ci_matrix(z, H, S, pairs, 1e-9)
    e, v = noci.generalized_eigh(H, S)
    vs = v.T @ S @ v
    assert float((vs - torch.eye(len(dets_a), device="cuda", dtype=torch.float64)).abs().max()) < 1e-9
    if energies_defined(z):
        assert np.abs(e.cpu().numpy() - z["noci_energies"]).max() < 1e-8


@pytest.mark.parametrize("name", NAMES)
def test_noci_full_calculation(name):
    z = load(name)
    eng = engine_for(z)
    out = noci.run(eng, str(z["excitations"]), reference="UHF", constrain_excited=True)
    e_hf = np.array([r.E for r in out["hf"]])
    assert all(r.converged for r in out["hf"])
    assert np.abs(e_hf - z["hf_energies"]).max() < 1e-7
    na, nb = int(z["n_alpha"]), int(z["n_beta"])
    dets_a, dets_b = out["dets_alpha"], out["dets_beta"]
    assert len(dets_a) == len(z["det_alpha"])
    H, S, pairs = noci.noci_matrix(eng, dets_a, dets_b, na, nb, return_pairs=True)
    # every element against the oracle on the GPU's own pairing of the GPU's orbitals
    from oracle import oracle
    ii, jj, a1, a2, b1, b2 = [t.cpu().numpy() for t in pairs]
    Hn, Sn = H.cpu().numpy(), S.cpu().numpy()
    for p in range(len(ii)):
        h, s = oracle.noci_element_paired(a1[p], a2[p], b1[p], b2[p], z["S"], z["H"], z["eri_dense"], na, nb,
                                          float(z["E_nuc"]))
        assert abs(h - Hn[ii[p], jj[p]]) < element_tolerance(a1[p], a2[p], b1[p], b2[p], z["S"], 1e-9)
        assert abs(s - Sn[ii[p], jj[p]]) < 1e-12
    # The reference stops its SCF on |dE| < 1e-11 alone; its MOM ground states keep
    # orbital-gradient residuals up to 3e-6 (max |F D S - S D F| of the fixture
    # orbitals), and off-diagonal NOCI elements are first order in that error.  The
    # GPU states converge the residual itself; the CI matrix from the reference's own
    # orbitals is checked to 1e-9 in test_ci_matrix_from_reference_determinants.
    if energies_defined(z):
        assert np.abs(out["energies"].cpu().numpy() - z["noci_energies"]).max() < 2e-5


def test_cli_noci_section(tmp_path):
    """Method = "NOCI" through the input-file runner (spin-flip singles on LiH)."""
    from pychem_gb300 import cli
    z = load("noci_lih_sfs_sto3g")
    coords = [[str(a), float(c), *map(float, x)] for a, c, x in zip(z["atoms"], z["charges"], z["coords_bohr"])]
    inp = tmp_path / "lih.inp"
    inp.write_text('[lih_sfs]\nMethod = "NOCI"\nBasis_Sets = ["STO-3G"]\nMultiplicity = 1\nCharge = 0\n'
                   'Coords_Units = "BOHR"\nCoords = %r\nReference = "UHF"\nConstrain_Excited = True\n'
                   'Excitations = "SFS"\n' % coords)
    res = cli.run_file(str(inp), stream=open("/dev/null", "w"))
    assert np.abs(np.array(res[0]["noci_energies"]) - z["noci_energies"]).max() < 1e-6
    assert (tmp_path / "lih_sfs.out").exists()
