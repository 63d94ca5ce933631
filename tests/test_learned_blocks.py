"""Host-side logic of the learned guess (no GPU): bond-frame slot maps, pair lists and
the assembly of pair and diagonal blocks into a density."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from pychem_gb300.learned import blocks as B
from pychem_gb300.learned.molgen import molecules
from pychem_gb300.ensemble import atom_table
from pychem_gb300.learned.train import TYPE_LIST, assemble
from pychem_gb300.molecule import Molecule


def _mols(n=6, seed=11):
    return [Molecule(c, "6-31G") for c in molecules(n, seed=seed)]


def _rot(seed):
    q, _ = np.linalg.qr(np.random.default_rng(seed).normal(size=(3, 3)))
    return q * np.sign(np.linalg.det(q))


@pytest.mark.parametrize("t", TYPE_LIST)
def test_slot_round_trip(t):
    g = torch.Generator().manual_seed(1)
    R = B.frames(torch.randn(40, 3, dtype=torch.float64, generator=g))
    par = torch.randn(40, B.NOFF, dtype=torch.float64, generator=g)
    back, mask = B.params_from_blocks(B.blocks_from_params(par, R, *t), R, *t)
    assert torch.allclose(back, par * mask, atol=1e-13)
    assert int(mask.sum()) == len(B.TYPES[t])


@pytest.mark.parametrize("ti", ["X", "H"])
def test_diagonal_corrections_symmetric_and_covariant(ti):
    """A correction is symmetric and turns with the bond: rotating the bond vector by Q
    maps the block to T(Q) block T(Q)^T."""
    g = torch.Generator().manual_seed(2)
    v = torch.randn(30, 3, dtype=torch.float64, generator=g)
    par = torch.randn(30, B.NDIAG, dtype=torch.float64, generator=g)
    blk = B.diag_from_params(par, B.frames(v), ti)
    assert torch.allclose(blk, blk.transpose(1, 2), atol=1e-14)
    Q = torch.as_tensor(_rot(3))
    blk_r = B.diag_from_params(par, B.frames(v @ Q.T), ti)
    TQ = B._Tmat(Q.expand(30, 3, 3), ti)
    assert torch.allclose(blk_r, TQ @ blk @ TQ.transpose(1, 2), atol=1e-12)


def test_pairs_match_brute_force():
    mols = _mols(8)
    at = atom_table(mols)
    pc = B.pairs(at, "cpu")
    got = set()
    for k in range(pc["mol"].numel()):
        m, gi, gj = int(pc["mol"][k]), int(pc["gi"][k]), int(pc["gj"][k])
        i, j = gi - at["atom0"][m], gj - at["atom0"][m]
        got.add((m, i, j))
        ti = "H" if mols[m].atoms[i][0] == "H" else "X"
        tj = "H" if mols[m].atoms[j][0] == "H" else "X"
        assert TYPE_LIST[int(pc["tc"][k])] == (ti, tj)
        assert int(pc["ao_i"][k]) == sum(B.nao_of(a[0]) for a in mols[m].atoms[:i])
        assert abs(float(pc["r"][k]) - np.linalg.norm(mols[m].atoms[j][2] - mols[m].atoms[i][2]) / B.TO_BOHR) < 1e-12
    want = set()
    for m, mol in enumerate(mols):
        for i, a in enumerate(mol.atoms):
            for j, b in enumerate(mol.atoms):
                if i != j and np.linalg.norm(a[2] - b[2]) / B.TO_BOHR <= B.CUTOFF:
                    want.add((m, i, j))
    assert got == want
    assert (np.diff(pc["mol"].numpy()) >= 0).all()


def test_assemble_reproduces_representable_blocks():
    """Pair blocks built from slot values in the i->j frame, their transposes in the
    j->i frame: assembling both orders gives back each block exactly, and the diagonal
    corrections of all neighbours are summed into the atom's own block."""
    mols = _mols(5, seed=4)
    n = max(m.NOrbitals for m in mols)
    pc = B.pairs(atom_table(mols), "cpu")
    P = pc["r"].numel()
    g = torch.Generator().manual_seed(5)
    R = B.frames(pc["vec"])
    D_true = torch.zeros(len(mols), n, n, dtype=torch.float64)
    par = torch.zeros(P, B.NPARAM, dtype=torch.float64)
    for k in range(P):
        m, ai, aj = int(pc["mol"][k]), int(pc["ao_i"][k]), int(pc["ao_j"][k])
        if ai > aj:
            continue
        t = TYPE_LIST[int(pc["tc"][k])]
        blk = B.blocks_from_params(torch.randn(1, B.NOFF, dtype=torch.float64, generator=g), R[k:k + 1], *t)[0]
        ni, nj = blk.shape
        D_true[m, ai:ai + ni, aj:aj + nj] = blk
        D_true[m, aj:aj + nj, ai:ai + ni] = blk.T
    for k in range(P):
        m, ai, aj = int(pc["mol"][k]), int(pc["ao_i"][k]), int(pc["ao_j"][k])
        t = TYPE_LIST[int(pc["tc"][k])]
        ni, nj = B.nao_of(t[0]), B.nao_of(t[1])
        p, mask = B.params_from_blocks(D_true[m, ai:ai + ni, aj:aj + nj][None], R[k:k + 1], *t)
        par[k, :B.NOFF] = p[0]
    dpar = torch.randn(P, B.NDIAG, dtype=torch.float64, generator=g)
    par[:, B.NOFF:] = dpar
    D = assemble(torch.zeros_like(D_true), pc, par)
    assert torch.allclose(D, D.transpose(1, 2), atol=1e-13)
    off = torch.ones_like(D, dtype=torch.bool)
    diag_want = torch.zeros_like(D)
    for k in range(P):
        m, ai = int(pc["mol"][k]), int(pc["ao_i"][k])
        t = TYPE_LIST[int(pc["tc"][k])]
        ni = B.nao_of(t[0])
        off[m, ai:ai + ni, ai:ai + ni] = False
        diag_want[m, ai:ai + ni, ai:ai + ni] += B.diag_from_params(dpar[k:k + 1], R[k:k + 1], t[0])[0]
    assert torch.allclose(D[off], D_true[off], atol=1e-12)
    assert torch.allclose(D[~off], diag_want[~off], atol=1e-12)
