"""Several basis sets and MO text files in the input-file runner, on CPU.

pychem_gb300.basis_fit against the reference's Methods/basis_fit.py outputs, and the
runner's bootstrap path (cli.run_bootstrap) driven with the oracle standing in for the
GPU engine and SCF: per-basis state energies against the reference's own multi-basis
runs (make_golden_bootstrap.py), Dump_MOs file names and contents, and the READ guess.
"""
import json
import os

import numpy as np
import pytest
import torch

from oracle import oracle
from pychem_gb300 import cli
from pychem_gb300.basis_fit import fit_orbitals
from pychem_gb300.molecule import Molecule
from pychem_gb300.scf import SCFResult

HERE = os.path.dirname(os.path.abspath(__file__))


def test_basis_fit_matches_reference():
    z = np.load(os.path.join(HERE, "golden", "basis_fit.npz"))
    names = sorted(set(k.rsplit("_", 1)[0] for k in z.files))
    assert len(names) == 5
    for n in names:
        old, new = z[n + "_meta"]
        coords = [[str(a), float(r[0]), *r[1:]] for a, r in zip(z[n + "_atoms"], z[n + "_coords"])]
        got = fit_orbitals(Molecule(coords, str(old)), z[n + "_C"], str(new))
        assert got.shape == z[n + "_fitted"].shape
        assert np.abs(got - z[n + "_fitted"]).max() < 1e-12, n


class OracleEngine:
    """CPU stand-in for a prepared GpuEngine: S, H, dense ERIs from the C oracle."""

    def __init__(self, mol):
        self.mol = mol
        atoms = [(a[0], a[1], *a[2]) for a in mol.atoms]
        b = oracle.Basis(atoms, mol.Basis)
        S, H = b.one_electron()
        self.S, self.H = torch.tensor(S), torch.tensor(H)
        self.eri = b.eri_dense()
        self.e_nuc = b.nuclear_repulsion()
        self.nbf = mol.NOrbitals


def oracle_rhf(eng, max_iter=128, D0=None, **kw):
    r = oracle.rhf(eng.S.numpy(), eng.H.numpy(), eng.eri, eng.mol.NAlphaElectrons, eng.e_nuc, max_iter=max_iter,
                   D0=None if D0 is None else D0.numpy())
    return SCFResult(E=r["E"], C=torch.tensor(r["C"]), eps=torch.tensor(r["eps"]), D=torch.tensor(r["D"]),
                     iterations=r["iterations"], converged=r["converged"])


def oracle_uhf(eng, cuhf=False, max_iter=300, C0=None, mom=False, d_tol=1e-8, cuhf_spaces=None, **kw):
    m = eng.mol
    c0 = None if C0 is None else (C0[0].numpy(), C0[1].numpy())
    r = oracle.uhf(eng.S.numpy(), eng.H.numpy(), eng.eri, m.NAlphaElectrons, m.NBetaElectrons, eng.e_nuc,
                   cuhf=cuhf, max_iter=max_iter, C0=c0, mom=mom, d_tol=d_tol, cuhf_spaces=cuhf_spaces)
    return SCFResult(E=r["E"], Ca=torch.tensor(r["Ca"]), Cb=torch.tensor(r["Cb"]), ea=torch.tensor(r["ea"]),
                     eb=torch.tensor(r["eb"]), Da=torch.tensor(r["Da"]), Db=torch.tensor(r["Db"]),
                     iterations=r["iterations"], converged=r["converged"])


@pytest.fixture
def oracle_runner(monkeypatch):
    monkeypatch.setattr(cli, "_engine", OracleEngine)
    monkeypatch.setattr(cli, "_rhf", oracle_rhf)
    monkeypatch.setattr(cli, "_uhf", oracle_uhf)
    return cli


def _opts(case):
    return {"METHOD": "HF", "REFERENCE": case["reference"], "BASIS_SETS": case["bases"],
            "COORDS": case["coords"], "CHARGE": 0, "MULTIPLICITY": 1, "MAX_SCF_ITERATIONS": 300,
            **({"EXCITATIONS": case["excitations"]} if case["excitations"] else {}),
            **({"CONSTRAIN_EXCITED": True} if case.get("constrain_excited") else {})}


with open(os.path.join(HERE, "golden", "bootstrap.json")) as _fh:
    BOOT = json.load(_fh)


BOOT_ORBITALS = np.load(os.path.join(HERE, "golden", "bootstrap.npz"))


def reference_residual(name, k, basis, coords, occ=None):
    """max |F D S - S D F| of the reference's final orbitals for call k (its SCF stops
    on |dE| alone; a large residual marks a state it left unconverged).  occ: the
    state's (n_alpha, n_beta), default the molecule's."""
    eng = OracleEngine(Molecule(coords, basis))
    S, H, eri = eng.S.numpy(), eng.H.numpy(), eng.eri
    na, nb = occ if occ is not None else (eng.mol.NAlphaElectrons, eng.mol.NBetaElectrons)
    Ca, Cb = BOOT_ORBITALS["%s_%d_alpha" % (name, k)], BOOT_ORBITALS["%s_%d_beta" % (name, k)]
    Da, Db = Ca[:, :na] @ Ca[:, :na].T, Cb[:, :nb] @ Cb[:, :nb].T
    J = np.einsum("cd,abcd->ab", Da + Db, eri)
    out = 0.0
    for D in (Da, Db):
        F = H + J - np.einsum("cb,abcd->ad", D, eri)
        out = max(out, float(np.abs(F @ D @ S - S @ D @ F).max()))
    return out


@pytest.mark.parametrize("name", [n for n in sorted(BOOT) if n.startswith("boot_")])
def test_bootstrap_energies_match_reference(name, oracle_runner, tmp_path):
    """Per-basis state energies against the reference's multi-basis run: ground states
    to 1e-8, MOM states (started from orbitals fitted with upstream's index
    bookkeeping) to 1e-5 where the reference converged them; upstream leaves some MOM
    states with orbital gradients near 1e-4 after 300 iterations, whose energies agree
    to 1e-3."""
    case = BOOT[name]
    res = oracle_runner.run_bootstrap(name, _opts(case), lambda line: None, str(tmp_path))
    got = [(pb["basis"], k, e) for pb in res["per_basis"] for k, e in enumerate(pb["E_hf"])]
    assert len(got) == len(case["calls"])
    for call, ((basis, k, e), (rb, rk, re_)) in enumerate(zip(got, case["calls"])):
        assert basis.replace("-", "").upper() == rb and k == rk
        if k == 0:
            assert abs(e - re_) < 1e-8, (basis, k, e, re_)
        else:
            converged = reference_residual(name, call, basis, case["coords"]) < 1e-5
            assert abs(e - re_) < (1e-5 if converged else 1e-3), (basis, k, e, re_)


def test_dump_and_read_mos(oracle_runner, tmp_path):
    """Dump_MOs writes <basis>_<state>.alpha_MOs / .beta_MOs as upstream; SCF_Guess =
    READ from them starts at the converged orbitals."""
    case = BOOT["boot_h2_mom_sto3g_631g"]
    opts = dict(_opts(case), DUMP_MOS=True)
    res = oracle_runner.run_bootstrap("dump", opts, lambda line: None, str(tmp_path))
    for basis in ("STO3G", "631G"):
        for k in (0, 1):
            for spin in ("alpha", "beta"):
                assert (tmp_path / ("%s_%d.%s_MOs" % (basis, k, spin))).exists()
    Ca = np.loadtxt(tmp_path / "631G_1.alpha_MOs")
    assert Ca.shape == (4, 4)
    opts = dict(_opts(case), BASIS_SETS=["6-31G"], SCF_GUESS="READ", MO_READ_BASIS="6-31G", MO_READ_STATE=[0, 1])
    again = oracle_runner.run_bootstrap("read", opts, lambda line: None, str(tmp_path))
    e_dump = res["per_basis"][1]["E_hf"]
    e_read = again["per_basis"][0]["E_hf"]
    assert abs(e_read[0] - e_dump[0]) < 1e-8 and abs(e_read[1] - e_dump[1]) < 1e-6
    assert again["per_basis"][0]["iterations"][0] <= 3


def test_read_guess_errors(oracle_runner, tmp_path):
    case = BOOT["boot_h2_mom_sto3g_631g"]
    opts = dict(_opts(case), BASIS_SETS=["6-31G"], SCF_GUESS="READ")
    with pytest.raises(ValueError):
        oracle_runner.run_bootstrap("x", opts, lambda line: None, str(tmp_path))
    opts.update(MO_READ_BASIS="6-31G", MO_READ_STATE=[0, 1])
    with pytest.raises(FileNotFoundError):
        oracle_runner.run_bootstrap("x", opts, lambda line: None, str(tmp_path))
    np.savetxt(tmp_path / "631G_0.alpha_MOs", np.eye(2))
    np.savetxt(tmp_path / "631G_0.beta_MOs", np.eye(2))
    with pytest.raises(ValueError):
        oracle_runner.run_bootstrap("x", opts, lambda line: None, str(tmp_path))


def test_mo_file_names():
    assert cli.mo_files("/w", "6-31G*", 2) == ("/w/631GS_2.alpha_MOs", "/w/631GS_2.beta_MOs")
    assert cli.mo_files(".", "cc-pVDZ", "0")[0].endswith("CCPVDZ_0.alpha_MOs")


def oracle_uhf_states(eng, cuhf=False, max_iter=300, e_tol=1e-10, d_tol=1e-8, C0=None, mom=False, occ=None,
                      cuhf_spaces=None):
    """The oracle's UHF with scf.uhf's signature (state occupation counts, CUHF spaces,
    occupied orbitals sorted by energy after MOM)."""
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
                     Da=torch.tensor(r["Da"]), Db=torch.tensor(r["Db"]), iterations=r["iterations"],
                     converged=r["converged"])


def _occupied_projector(C, n, S):
    Co = C[:, :n]
    return Co @ Co.T @ S


@pytest.mark.parametrize("name", [n for n in sorted(BOOT) if n.startswith("states_")])
def test_excitation_keyword_states_match_reference(name, monkeypatch, tmp_path):
    """Method = HF with excitation keywords other than HOMO-LUMO.  The runner's states
    (noci.excited_states + noci.hf_states, the oracle standing in for the GPU UHF) go
    against the reference's own state energies.

    Upstream starts each state from its predecessor's final orbitals reordered by
    column index (pychem.py:90-93).  After MOM the virtual columns are ordered by tiny
    overlap sums (mom.py:24-33), so deeper in the chain the start can depend on
    rounding.  Each state whose starting occupied space equals the reference's, rebuilt
    from the reference's recorded orbitals, is compared: 1e-8 from the core guess,
    1e-5 where the reference converged the MOM state, 1e-3 where it left orbital
    gradients above 1e-5.  At least the first excited state of every list qualifies."""
    from pychem_gb300 import noci
    case = BOOT[name]
    monkeypatch.setattr(cli, "_engine", OracleEngine)
    monkeypatch.setattr(noci, "uhf", oracle_uhf_states)
    res = cli.run_section(name, _opts(case), lambda line: None, str(tmp_path))
    mol = Molecule(case["coords"], case["bases"][0])
    eng = OracleEngine(mol)
    S = eng.S.numpy()
    lists, _ = noci.excited_states(mol.NAlphaElectrons, mol.NBetaElectrons, mol.NOrbitals, case["excitations"],
                                   n_core=noci.n_core_orbitals([int(a[1]) for a in case["coords"]]))
    spin_flip = "SF" in case["excitations"]
    ours = noci.hf_states(eng, lists, spin_flip=spin_flip, reference="UHF",
                          constrain_excited=bool(case.get("constrain_excited")))
    got = [st["E_hf"] for st in res["states"]]
    assert len(got) == len(case["calls"]) == len(lists)
    assert np.allclose(got, [r.E for r in ours], atol=1e-10)
    order = [c[1] for c in case["calls"]]
    compared = 0
    for call, (basis, k, e_ref) in enumerate(case["calls"]):
        na, nb = sum(lists[k][0]), sum(lists[k][1])
        if call == 0:
            assert abs(got[k] - e_ref) < 1e-8, (k, got[k], e_ref)
            compared += 1
            continue
        prev = order[call - 1]
        if spin_flip:
            same = True          # both spins from the predecessor's alpha orbitals, no reordering
        else:
            ref_a = noci.reorder_mos(torch.tensor(BOOT_ORBITALS["%s_%d_alpha" % (name, call - 1)]), lists[k][0])
            ref_b = noci.reorder_mos(torch.tensor(BOOT_ORBITALS["%s_%d_beta" % (name, call - 1)]), lists[k][1])
            our_a = noci.reorder_mos(ours[prev].Ca, lists[k][0])
            our_b = noci.reorder_mos(ours[prev].Cb, lists[k][1])
            same = all(np.abs(_occupied_projector(x.numpy(), n, S) - _occupied_projector(y.numpy(), n, S)).max()
                       < 1e-4 for x, y, n in ((ref_a, our_a, na), (ref_b, our_b, nb)))
        if not same:
            continue
        tol = 1e-5 if reference_residual(name, call, basis_name(basis), case["coords"], (na, nb)) < 1e-5 else 1e-3
        assert abs(got[k] - e_ref) < tol, (k, got[k], e_ref)
        compared += 1
    print("%s: %d of %d states compared" % (name, compared, len(lists)))
    assert compared >= 2


def basis_name(clean):
    return {"STO3G": "STO-3G", "631G": "6-31G", "CCPVDZ": "cc-pVDZ"}[clean]


def test_rhf_sections_that_need_unrestricted_states(monkeypatch, tmp_path):
    """Upstream's Reference = RHF only changes its printout; its SCF is unrestricted.
    An RHF section with excited states (H2 HOMO-LUMO) or an open shell (OH) gives the
    reference's UHF energies (h2_mom_631g, oh_uhf_631g fixtures)."""
    monkeypatch.setattr(cli, "_engine", OracleEngine)
    monkeypatch.setattr(cli, "uhf", oracle_uhf)
    g = np.load(os.path.join(HERE, "golden", "h2_mom_631g.npz"))
    coords = [[str(a), float(z), *map(float, x)] for a, z, x in zip(g["atoms"], g["charges"], g["coords_bohr"])]
    opts = {"METHOD": "HF", "REFERENCE": "RHF", "BASIS_SETS": ["6-31G"], "COORDS": coords, "COORDS_UNITS": "BOHR",
            "EXCITATIONS": "HOMO-LUMO"}
    lines = []
    res = cli.run_section("h2", opts, lines.append, str(tmp_path))
    assert any("unrestricted" in ln for ln in lines)
    e = [st["E_hf"] for st in res["states"]]
    assert abs(e[0] - float(g["E_ground"])) < 1e-8 and abs(e[1] - float(g["E_excited"])) < 1e-6
    o = np.load(os.path.join(HERE, "golden", "oh_uhf_631g.npz"))
    coords = [[str(a), float(z), *map(float, x)] for a, z, x in zip(o["atoms"], o["charges"], o["coords_bohr"])]
    opts = {"METHOD": "HF", "REFERENCE": "RHF", "BASIS_SETS": ["6-31G"], "COORDS": coords, "COORDS_UNITS": "BOHR",
            "MULTIPLICITY": 2}
    res = cli.run_section("oh", opts, lambda line: None, str(tmp_path))
    assert abs(res["states"][0]["E_hf"] - float(o["E_scf"])) < 1e-8


def test_noci_then_scattering_section(monkeypatch, tmp_path):
    """Method = NOCI with Job_Type = PROPERTY through the runner (make_golden_noci_property.py:
    H2 / 6-31G, ground and HOMO -> LUMO states): NOCI energies and the scattering table
    over the NOCI states against the reference, with the oracle standing in for the GPU
    integrals, UHF, eigensolver and intensity evaluation."""
    from scipy.linalg import eigh
    from pychem_gb300 import noci, scattering

    with open(os.path.join(HERE, "golden", "noci_property.json")) as fh:
        ref = json.load(fh)

    class Engine(OracleEngine):
        def coulomb_exchange(self, W):
            E = torch.tensor(self.eri)
            return torch.einsum("ncd,abcd->nab", W, E), torch.einsum("ncb,abcd->nad", W, E)

    def gen_eigh(H, S):
        e, v = eigh(H.numpy(), S.numpy())
        return torch.tensor(e), torch.tensor(v)

    def intensities(mol, grid, densities):
        b = oracle.Basis([(a[0], a[1], *a[2]) for a in mol.atoms], mol.Basis)
        return np.array([[oracle.scattering_intensity(np.asarray(a), np.asarray(c), b.eri_dense(scattering=s),
                                                      mol.NElectrons) for a, c in densities] for s in grid])

    monkeypatch.setattr(cli, "_engine", Engine)
    monkeypatch.setattr(noci, "uhf", oracle_uhf_states)
    monkeypatch.setattr(noci, "generalized_eigh", gen_eigh)
    monkeypatch.setattr(scattering, "intensities", intensities)
    opts = {"METHOD": "NOCI", "REFERENCE": "UHF", "BASIS_SETS": [ref["basis"]], "COORDS": ref["coords"],
            "EXCITATIONS": ref["excitations"], "CONSTRAIN_EXCITED": True, "JOB_TYPE": "PROPERTY",
            "PROPERTY_TYPE": "SCATTERING", "PROPERTY_GRID": ref["grid"]}
    res = cli.run_section("h2", opts, lambda line: None, str(tmp_path))
    assert np.abs(np.array(res["noci_energies"]) - ref["noci_energies"]).max() < 1e-6
    assert np.abs(np.array(res["scattering"]["intensities"]) - np.array(ref["intensities"])).max() < 1e-6


def _cpu_ump2(eng, res, scale=None):
    """scf.ump2's stand-in on CPU: the oracle's UMP2 over its dense ERI tensor."""
    m = eng.mol
    return oracle.ump2(*(np.asarray(t.cpu() if hasattr(t, "cpu") else t) for t in (res.Ca, res.Cb, res.ea, res.eb)),
                       eng.eri, m.NAlphaElectrons, m.NBetaElectrons, scale=scale)


with open(os.path.join(HERE, "golden", "mp2_states.json")) as _fh:
    MP2_STATES = json.load(_fh)


MP2_STATE_ORBITALS = np.load(os.path.join(HERE, "golden", "mp2_states.npz"))


def _state_residual(eng, Ca, Cb, occ_a, occ_b, cuhf):
    """max |F D S - S D F| of a state's orbitals (occupied columns first), with the
    CUHF constraint of its occupancy when cuhf."""
    S, H, eri = eng.S.numpy(), eng.H.numpy(), eng.eri
    na, nb = sum(occ_a), sum(occ_b)
    Da, Db = Ca[:, :na] @ Ca[:, :na].T, Cb[:, :nb] @ Cb[:, :nb].T
    J = np.einsum("cd,abcd->ab", Da + Db, eri)
    Fa = H + J - np.einsum("cb,abcd->ad", Da, eri)
    Fb = H + J - np.einsum("cb,abcd->ad", Db, eri)
    if cuhf:
        tot = [a + b for a, b in zip(occ_a, occ_b)]
        Fa, Fb = oracle.cuhf_constraint(S, Da, Db, Fa, Fb, na, nb, (tot.count(2), tot.count(1)))
    return max(float(np.abs(F @ D @ S - S @ D @ F).max()) for F, D in ((Fa, Da), (Fb, Db)))


@pytest.mark.parametrize("name", sorted(MP2_STATES))
def test_mp2_over_excited_states(name, monkeypatch, tmp_path):
    """Method = MP2 with Excitations = HOMO-LUMO through the runner (UHF: the MOM
    branch; CUHF: the state loop with the occupancy's constraint spaces), MP2 of every
    state from its own orbitals and orbital energies, against the reference's printed
    per-state totals (make_golden_mp2_states.py): 1e-8 / 1e-6 where the reference's
    state is stationary (orbital gradient below 1e-5), 1e-3 where it stopped short."""
    from pychem_gb300 import noci
    case = MP2_STATES[name]
    monkeypatch.setattr(cli, "_engine", OracleEngine)
    monkeypatch.setattr(cli, "uhf", oracle_uhf)
    monkeypatch.setattr(noci, "uhf", oracle_uhf_states)
    monkeypatch.setattr(cli, "ump2", _cpu_ump2)
    opts = {"METHOD": "MP2", "REFERENCE": case["reference"], "BASIS_SETS": [case["basis"]],
            "COORDS": case["coords"], "EXCITATIONS": "HOMO-LUMO", "MAX_SCF_ITERATIONS": 300}
    res = cli.run_section(name, opts, lambda line: None, str(tmp_path))
    assert len(res["states"]) == 2
    mol = Molecule(case["coords"], case["basis"])
    eng = OracleEngine(mol)
    lists, _ = noci.excited_states(mol.NAlphaElectrons, mol.NBetaElectrons, mol.NOrbitals, "HOMO-LUMO")
    for k, st in enumerate(res["states"]):
        stationary = _state_residual(eng, MP2_STATE_ORBITALS["%s_%d_alpha" % (name, k)],
                                     MP2_STATE_ORBITALS["%s_%d_beta" % (name, k)], lists[k][0], lists[k][1],
                                     case["reference"] == "CUHF") < 1e-5
        e_ref, m_ref = case["E_hf"][k], case["E_mp2_total"][k]
        assert abs(st["E_hf"] - e_ref) < ((1e-8 if k == 0 else 1e-6) if stationary else 1e-3), (k, st["E_hf"], e_ref)
        assert abs(st["E_hf"] + st["E_mp2_corr"] - m_ref) < (1e-6 if stationary else 1e-3), (k, m_ref)
