"""NOCI on CPU: the oracle pinned to the reference's CI matrices, and the host logic of
pychem_gb300.noci (state lists, spin-flip determinants, CI-matrix assembly with a dense
einsum standing in for the GPU digestion) against the same fixtures.

Fixtures: tests/golden/noci_*.npz from make_golden_noci.py.  Some upstream elements
are not defined by the orbitals: with two zero overlaps in one spin the two-zero form
(Methods/noci.py:279-300) reads one pair out of a degenerate null space, and a
zero-overlap pair whose plain dot product vanishes gets its phase from rounding noise
(noci.py:199-203).  pychem_gb300.noci fixes both choices canonically; such elements are
compared with the oracle evaluated on the same paired orbitals, every other element
with the reference's value.
"""
import glob
import os

import numpy as np
import pytest
import torch

from oracle import oracle
from pychem_gb300 import noci

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = sorted(glob.glob(os.path.join(HERE, "golden", "noci_*.npz")))
NAMES = [os.path.basename(c)[:-4] for c in CASES]


def load(name):
    return np.load(os.path.join(HERE, "golden", name + ".npz"))


_MASKS = {}


def basis_dependent(z):
    """Mask of CI elements that the upstream algorithm leaves to arbitrary choices:
    two zero overlaps in one spin, a zero pair whose plain dot product vanishes, or a
    value that moves under 1e-12 perturbations of the determinants (oracle, reference
    pairing)."""
    key = (str(z["excitations"]), float(z["E_nuc"]))
    if key in _MASKS:
        return _MASKS[key]
    na, nb = int(z["n_alpha"]), int(z["n_beta"])
    S = z["S"]
    m = len(z["det_alpha"])
    mask = np.zeros((m, m), dtype=bool)
    for i in range(m):
        for j in range(i + 1):
            a1, a2 = oracle.noci_biorthogonalize(z["det_alpha"][i], z["det_alpha"][j], S, na)
            b1, b2 = oracle.noci_biorthogonalize(z["det_beta"][i], z["det_beta"][j], S, nb)
            za, zb = oracle.noci_zero_counts(a1, a2, b1, b2, S)
            bad = za >= 2 or zb >= 2
            for x1, x2 in ((a1, a2), (b1, b2)):
                ov = np.einsum("pi,pq,qi->i", x1, S, x2)
                dot = np.einsum("pi,pi->i", x1, x2)
                bad |= bool(np.any((np.abs(ov) <= oracle.NOCI_THRESH) & (np.abs(dot) <= 1e-8)))
            mask[i, j] = mask[j, i] = bad
    rng = np.random.default_rng(3)
    args = (S, z["H"], z["eri_dense"], na, nb, float(z["E_nuc"]))
    H0 = oracle.noci(list(z["det_alpha"]), list(z["det_beta"]), *args)[2]
    for _ in range(2):
        da = [x + 1e-12 * rng.standard_normal(x.shape) for x in z["det_alpha"]]
        db = [x + 1e-12 * rng.standard_normal(x.shape) for x in z["det_beta"]]
        mask |= np.abs(oracle.noci(da, db, *args)[2] - H0) > 1e-8
    _MASKS[key] = mask
    return mask


_DEFINED = {}


def energies_defined(z):
    """Whether the upstream algorithm's NOCI energies are a function of the orbitals:
    the oracle's energies move by less than 1e-8 under 1e-12 perturbations of the
    determinants.  On the spin-flip CISD lists with doubles they move by up to 0.04 Eh
    (elements left to arbitrary choices), so the reference's values there are not
    reproducible by any implementation."""
    key = (str(z["excitations"]), float(z["E_nuc"]))
    if key not in _DEFINED:
        na, nb = int(z["n_alpha"]), int(z["n_beta"])
        args = (z["S"], z["H"], z["eri_dense"], na, nb, float(z["E_nuc"]))
        e0 = oracle.noci(list(z["det_alpha"]), list(z["det_beta"]), *args)[0]
        rng = np.random.default_rng(4)
        spread = 0.0
        for _ in range(2):
            da = [x + 1e-12 * rng.standard_normal(x.shape) for x in z["det_alpha"]]
            db = [x + 1e-12 * rng.standard_normal(x.shape) for x in z["det_beta"]]
            spread = max(spread, float(np.abs(oracle.noci(da, db, *args)[0] - e0).max()))
        _DEFINED[key] = spread < 1e-8
    return _DEFINED[key]


def test_fixtures_present():
    assert len(CASES) >= 7


@pytest.mark.parametrize("name", NAMES)
def test_oracle_noci_matches_reference(name):
    z = load(name)
    e, v, H, S = oracle.noci(list(z["det_alpha"]), list(z["det_beta"]), z["S"], z["H"], z["eri_dense"],
                             int(z["n_alpha"]), int(z["n_beta"]), float(z["E_nuc"]))
    mask = basis_dependent(z)
    assert np.abs(S - z["ci_S"]).max() < 1e-12
    assert np.abs(np.where(mask, 0.0, H - z["ci_H"])).max() < 1e-9
    if energies_defined(z):
        assert np.abs(e - z["noci_energies"]).max() < 1e-9


@pytest.mark.parametrize("name", NAMES)
def test_oracle_assemble_matches_reference(name):
    z = load(name)
    for k, (idx, oa, ob) in enumerate(zip(z["sf_index"], z["sf_alpha"], z["sf_beta"])):
        C, occ = z["hf_alpha"][idx], z["hf_occ_alpha"][idx]
        assert np.array_equal(oracle.noci_assemble(oa, C, occ), z["det_alpha"][k])
        assert np.array_equal(oracle.noci_assemble(ob, C, occ), z["det_beta"][k])


@pytest.mark.parametrize("name", NAMES)
def test_state_lists_match_reference(name):
    z = load(name)
    na, nb, norb = int(z["n_alpha"]), int(z["n_beta"]), z["S"].shape[0]
    states, sf = noci.excited_states(na, nb, norb, str(z["excitations"]))
    assert [s[0] for s in states] == z["hf_occ_alpha"].tolist()
    assert [s[1] for s in states] == z["hf_occ_beta"].tolist()
    assert [s[0] for s in sf] == z["sf_index"].tolist()
    assert [s[1] for s in sf] == z["sf_alpha"].tolist()
    assert [s[2] for s in sf] == z["sf_beta"].tolist()


@pytest.mark.parametrize("name", NAMES)
def test_determinants_match_reference(name):
    z = load(name)
    na, nb, norb = int(z["n_alpha"]), int(z["n_beta"]), z["S"].shape[0]
    states, sf = noci.excited_states(na, nb, norb, str(z["excitations"]))

    class R:
        pass
    res = []
    for k in range(len(states)):
        r = R()
        r.Ca, r.Cb = torch.tensor(z["hf_alpha"][k]), torch.tensor(z["hf_beta"][k])
        res.append(r)
    da, db = noci.determinants(states, res, sf)
    assert len(da) == len(z["det_alpha"])
    for a, b, ra, rb in zip(da, db, z["det_alpha"], z["det_beta"]):
        assert torch.equal(a, torch.tensor(ra)) and torch.equal(b, torch.tensor(rb))


class _Mol:
    def __init__(self, e, na, nb):
        self.e = e
        self.NAlphaElectrons, self.NBetaElectrons = na, nb

    def nuclear_repulsion(self):
        return self.e


class DenseEngine:
    """CPU stand-in for GpuEngine in the CI-matrix assembly: S, H and J/K by einsum on
    the fixture's dense ERI tensor."""

    def __init__(self, z):
        self.S, self.H = torch.tensor(z["S"]), torch.tensor(z["H"])
        self.eri = torch.tensor(z["eri_dense"])
        self.mol = _Mol(float(z["E_nuc"]), int(z["n_alpha"]), int(z["n_beta"]))
        self.nbf = self.S.shape[0]

    def coulomb_exchange(self, W):
        return torch.einsum("ncd,abcd->nab", W, self.eri), torch.einsum("ncb,abcd->nad", W, self.eri)


def element_tolerance(a1, a2, b1, b2, S, tol):
    """tol, widened for nearly orthogonal pairs: the element divides by each paired
    overlap above the zero threshold, so roundoff grows like 1/min(overlap)."""
    ov = np.concatenate([np.diagonal(a1.T @ S @ a2), np.diagonal(b1.T @ S @ b2)])
    kept = ov[ov > oracle.NOCI_THRESH]
    return tol + (1e-15 / kept.min() if kept.size else 0.0)


def check_ci_matrix(z, H, S, pairs, tol):
    """H, S against the reference outside basis-dependent elements, and every element
    against the oracle on the same paired orbitals."""
    na, nb = int(z["n_alpha"]), int(z["n_beta"])
    mask = basis_dependent(z)
    H, S = H.cpu().numpy(), S.cpu().numpy()
    # overlaps through a zero pair (below 1e-8) carry that pair's arbitrary sign
    assert np.abs(np.abs(S) - np.abs(z["ci_S"])).max() < 1e-12
    assert np.abs(np.where(np.abs(z["ci_S"]) > 1e-8, S - z["ci_S"], 0.0)).max() < 1e-12
    assert np.abs(np.where(mask, 0.0, H - z["ci_H"])).max() < tol
    ii, jj, a1, a2, b1, b2 = [t.cpu().numpy() for t in pairs]
    for p in range(len(ii)):
        h, s = oracle.noci_element_paired(a1[p], a2[p], b1[p], b2[p], z["S"], z["H"], z["eri_dense"], na, nb,
                                          float(z["E_nuc"]))
        assert abs(h - H[ii[p], jj[p]]) < element_tolerance(a1[p], a2[p], b1[p], b2[p], z["S"], tol), (ii[p], jj[p])
        assert abs(s - S[ii[p], jj[p]]) < 1e-12


@pytest.mark.parametrize("name", NAMES)
def test_ci_matrix_assembly(name):
    z = load(name)
    dets_a = [torch.tensor(x) for x in z["det_alpha"]]
    dets_b = [torch.tensor(x) for x in z["det_beta"]]
    H, S, pairs = noci.noci_matrix(DenseEngine(z), dets_a, dets_b, int(z["n_alpha"]), int(z["n_beta"]),
                                   return_pairs=True)
    check_ci_matrix(z, H, S, pairs, 1e-9)
    if energies_defined(z):
        from scipy.linalg import eigh
        e = eigh(H.numpy(), S.numpy(), eigvals_only=True)
        assert np.abs(e - z["noci_energies"]).max() < 1e-9


def test_core_orbital_counts():
    assert noci.n_core_orbitals([3, 1]) == 1
    assert noci.n_core_orbitals([8, 1, 1]) == 1
    assert noci.n_core_orbitals([17, 11]) == 10
    assert noci.n_core_orbitals([1, 2]) == 0


def test_excitation_lists():
    # HOMO-LUMO adds one alpha single; S adds every single of each spin above the core
    states, sf = noci.excited_states(3, 3, 6, "HOMO-LUMO")
    assert states == [([1, 1, 1, 0, 0, 0], [1, 1, 1, 0, 0, 0]), ([1, 1, 0, 1, 0, 0], [1, 1, 1, 0, 0, 0])]
    assert sf == []
    states, _ = noci.excited_states(2, 2, 4, "SINGLES", n_core=1)
    assert len(states) == 1 + 2 + 2
    assert states[1] == ([1, 0, 1, 0], [1, 1, 0, 0])
    states, _ = noci.excited_states(2, 2, 4, "SD", n_core=0)
    # 4 + 4 singles, 16 alpha x beta pairs, one double per spin
    assert len(states) == 1 + 8 + 16 + 2
    with pytest.raises(ValueError):
        noci.excited_states(2, 2, 4, "TRIPLES")


def test_reorder_mos():
    C = torch.arange(16.0).view(4, 4)
    out = noci.reorder_mos(C, [1, 0, 1, 0])
    assert torch.equal(out[:, 1], C[:, 2]) and torch.equal(out[:, 2], C[:, 1])
    assert torch.equal(noci.reorder_mos(C, [1, 1, 0, 0]), C)


def test_spin_flip_lists_without_ci_fail_like_the_reference():
    """Upstream's plain SFD list names a third Hartree-Fock state that its state list
    lacks (IndexError) and its SFSD list asks for orbitals the high-spin states leave
    empty (ValueError in noci.assemble_orbitals); both fail the same way here."""
    class R:
        pass

    for exc, err in (("SFD", IndexError), ("SFSD", ValueError)):
        states, sf = noci.excited_states(2, 2, 6, exc)
        res = []
        for _ in states:
            r = R()
            r.Ca = r.Cb = torch.eye(6, dtype=torch.float64)
            res.append(r)
        with pytest.raises(err):
            noci.determinants(states, res, sf)


@pytest.mark.parametrize("name", ["noci_c2_sfd_cisd_631g", "noci_lih_sfd_cisd_sto3g", "noci_lih_sfsd_cisd_sto3g"])
def test_ci_matrix_is_continuous_in_the_orbitals(name):
    """Canonical pairing: 1e-13 noise on the determinants moves no CI element by more
    than 1e-8 (the upstream choices move some by up to 0.3 Eh on these lists)."""
    z = load(name)
    eng = DenseEngine(z)
    na, nb = int(z["n_alpha"]), int(z["n_beta"])
    da = [torch.tensor(x) for x in z["det_alpha"]]
    db = [torch.tensor(x) for x in z["det_beta"]]
    H0, S0 = noci.noci_matrix(eng, da, db, na, nb)
    g = torch.Generator().manual_seed(5)
    for _ in range(3):
        pa = [x + 1e-13 * torch.randn(x.shape, generator=g, dtype=torch.float64) for x in da]
        pb = [x + 1e-13 * torch.randn(x.shape, generator=g, dtype=torch.float64) for x in db]
        H1, S1 = noci.noci_matrix(eng, pa, pb, na, nb)
        assert float((H1 - H0).abs().max()) < 1e-8
        assert float((S1 - S0).abs().max()) < 1e-10


def _excitation_cases():
    import json
    with open(os.path.join(HERE, "golden", "excitation_lists.json")) as fh:
        return json.load(fh)


@pytest.mark.parametrize("case", _excitation_cases(),
                         ids=lambda c: "%s-%s" % (c["molecule"], c["excitations"] or "custom"))
def test_excitation_lists_match_reference(case):
    """Every upstream excitation keyword on closed- and open-shell molecules
    (make_golden_excitations.py): the state occupancies, the spin-flip list and the
    core-orbital count; custom lists are rejected as upstream rejects them."""
    if case.get("rejected"):
        with pytest.raises(ValueError):
            noci.excited_states(2, 2, 8, case["excitations"], alpha_excitations=case["alpha_excitations"],
                                beta_excitations=case["beta_excitations"])
        return
    n_core = noci.n_core_orbitals([int(z) for z in case["charges"]])
    assert n_core == case["n_core"]
    states, sf = noci.excited_states(case["n_alpha"], case["n_beta"], case["n_orbitals"], case["excitations"],
                                     n_core=n_core)
    assert [[list(a), list(b)] for a, b in states] == case["states"]
    assert [[i, list(a), list(b)] for i, a, b in sf] == case["spin_flip"]


def _oracle_uhf_for(z):
    """The oracle's UHF in place of scf.uhf, with the occupation counts, starting
    orbitals and CUHF spaces that hf_states passes."""
    from pychem_gb300.scf import SCFResult
    S, H, eri, e_nuc = z["S"], z["H"], z["eri_dense"], float(z["E_nuc"])

    def uhf(engine, cuhf=False, max_iter=300, e_tol=1e-10, d_tol=1e-8, C0=None, mom=False, occ=None,
            cuhf_spaces=None):
        na, nb = occ
        c0 = None if C0 is None else (C0[0].numpy(), C0[1].numpy())
        r = oracle.uhf(S, H, eri, na, nb, e_nuc, cuhf=cuhf, max_iter=max_iter, d_tol=d_tol, C0=c0, mom=mom,
                       cuhf_spaces=cuhf_spaces)
        Ca, Cb, ea, eb = r["Ca"], r["Cb"], r["ea"], r["eb"]
        if mom:                                  # occupied orbitals by energy, as scf.uhf
            for C, e, n in ((Ca, ea, na), (Cb, eb, nb)):
                idx = np.argsort(e[:n], kind="stable")
                C[:, :n], e[:n] = C[:, :n][:, idx], e[:n][idx]
        return SCFResult(E=r["E"], Ca=torch.tensor(Ca), Cb=torch.tensor(Cb), ea=torch.tensor(ea),
                         eb=torch.tensor(eb), iterations=r["iterations"], converged=r["converged"])
    return uhf


@pytest.mark.parametrize("name", NAMES)
def test_state_scf_orchestration_against_reference(name, monkeypatch):
    """noci.hf_states (state order, starting orbitals, MOM, constraints), determinants
    and noci_matrix with the oracle's UHF and dense J/K: the reference's state
    energies to 1e-7 and, where its algorithm defines them, its NOCI energies to 2e-5
    (its MOM states stop on |dE| alone)."""
    from scipy.linalg import eigh
    z = load(name)
    monkeypatch.setattr(noci, "uhf", _oracle_uhf_for(z))
    eng = DenseEngine(z)
    na, nb = int(z["n_alpha"]), int(z["n_beta"])
    exc = str(z["excitations"])
    states, sf = noci.excited_states(na, nb, z["S"].shape[0], exc)
    res = noci.hf_states(eng, states, spin_flip="SF" in exc, reference="UHF", constrain_excited=True)
    assert np.abs(np.array([r.E for r in res]) - z["hf_energies"]).max() < 1e-7
    da, db = noci.determinants(states, res, sf if "SF" in exc else [])
    H, S = noci.noci_matrix(eng, da, db, na, nb)
    if energies_defined(z):
        e = eigh(H.numpy(), S.numpy(), eigvals_only=True)
        assert np.abs(e - z["noci_energies"]).max() < 2e-5


def test_ci_matrix_in_chunks_equals_one_pass():
    """noci_matrix evaluates pairs in bounded chunks; any chunking gives the same
    matrices and paired orbitals."""
    z = load("noci_c2_sfd_cisd_631g")
    eng = DenseEngine(z)
    na, nb = int(z["n_alpha"]), int(z["n_beta"])
    da = [torch.tensor(x) for x in z["det_alpha"]]
    db = [torch.tensor(x) for x in z["det_beta"]]
    H1, S1, p1 = noci.noci_matrix(eng, da, db, na, nb, return_pairs=True)
    H2, S2, p2 = noci.noci_matrix(eng, da, db, na, nb, return_pairs=True, max_pairs=37)
    assert float((H1 - H2).abs().max()) < 1e-12 and float((S1 - S2).abs().max()) < 1e-14
    for x, y in zip(p1, p2):
        assert x.shape == y.shape and float((x.double() - y.double()).abs().max()) < 1e-12


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_ci_matrix_random_determinants(seed):
    """Random S-orthonormal orbital sets on LiH / 6-31G integrals, some built to share
    or exclude occupied orbitals (exact zero overlaps in one or both spins, unequal
    alpha and beta counts): every element against the oracle on the same pairing."""
    z = load("noci_lih_sfs_631g")
    S = z["S"]
    n = S.shape[0]
    rng = np.random.default_rng(seed)
    s, U = np.linalg.eigh(S)
    X = U / np.sqrt(s)                                   # S-orthonormal basis

    def orbitals():
        Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
        return X @ Q

    base = orbitals()
    swap14 = base.copy()
    swap14[:, [1, 4]] = swap14[:, [4, 1]]                # one alpha zero against base
    swap_both = base.copy()
    swap_both[:, [0, 1, 2, 3]] = swap_both[:, [2, 3, 0, 1]]   # two alpha zeros and a beta zero
    rnd = orbitals()
    rnd_swap = rnd.copy()
    rnd_swap[:, [1, 4]] = rnd_swap[:, [4, 1]]
    alphas = [base, orbitals(), rnd_swap, swap14, base, swap_both]
    betas = [base, orbitals(), rnd_swap, swap14, base[:, ::-1].copy(), swap_both]   # 4: a beta zero
    dets_a = [torch.tensor(c) for c in alphas]
    dets_b = [torch.tensor(c) for c in betas]
    na, nb = 2, 1
    zeng = DenseEngine(z)
    H, Sm, pairs = noci.noci_matrix(zeng, dets_a, dets_b, na, nb, return_pairs=True)
    ii, jj, a1, a2, b1, b2 = [t.numpy() for t in pairs]
    zeros = set()
    for p in range(len(ii)):
        zeros.add(oracle.noci_zero_counts(a1[p], a2[p], b1[p], b2[p], S))
        h, ov = oracle.noci_element_paired(a1[p], a2[p], b1[p], b2[p], S, z["H"], z["eri_dense"], na, nb,
                                           float(z["E_nuc"]))
        assert abs(h - H[ii[p], jj[p]].item()) < element_tolerance(a1[p], a2[p], b1[p], b2[p], S, 1e-9)
        assert abs(ov - Sm[ii[p], jj[p]].item()) < 1e-12
    assert torch.allclose(H, H.T) and torch.allclose(Sm, Sm.T)
    assert {(0, 0), (1, 0), (0, 1), (2, 1)} <= zeros      # every element form occurs
