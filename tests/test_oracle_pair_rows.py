"""The compact pair tensor of the MP2 path (GpuEngine.stored_pair_map) gives no row to
an AO pair whose shell pair is in no off-diagonal stored quartet.  Such a shell pair P
has Q_P Q_X <= 1e-8 for every pair X (the upstream screen, Methods/hartree_fock.py:
244-312), so its only stored quartet is its own diagonal one, bounded by
Q_P^2 <= (1e-8 / max Q)^2.  Checked here on the oracle for a four-water cluster: the
bound, and the MP2 energy with those pairs' rows and columns removed against the full
tensor."""
import numpy as np
import pytest

from oracle import oracle
from pychem_gb300 import workloads as W
from pychem_gb300.molecule import Molecule


@pytest.fixture(scope="module")
def water4():
    mol = Molecule(W.water_cluster(nx=2, ny=2, nz=1), "6-31G")
    b = oracle.Basis([(a[0], a[1], *a[2]) for a in mol.atoms], "6-31G")
    return mol, b


def _unused_shell_pairs(b, Q):
    qa = b.quartet_array(Q)
    off = qa[(qa[:, 0] != qa[:, 2]) | (qa[:, 1] != qa[:, 3])]
    used = set(map(tuple, off[:, :2])) | set(map(tuple, off[:, 2:]))
    ia, ib = np.triu_indices(b.nshell)
    return [(int(a), int(c)) for a, c in zip(ia, ib) if (a, c) not in used]


def test_unused_pairs_fail_every_schwarz_test(water4):
    _, b = water4
    Q = b.schwarz()
    unused = _unused_shell_pairs(b, Q)
    assert len(unused) > 0                          # the cluster has far pairs
    for a, c in unused:
        assert Q[a, c] * Q.max() <= oracle.INTEGRAL_THRESHOLD
        assert Q[a, c] ** 2 <= (oracle.INTEGRAL_THRESHOLD / Q.max()) ** 2


def test_mp2_without_unused_pair_rows(water4):
    mol, b = water4
    Q = b.schwarz()
    unused = _unused_shell_pairs(b, Q)
    sh_of = np.concatenate([np.full(2 * s[0] + 1, k) for k, s in enumerate(b.shells)])
    lo = np.minimum.outer(sh_of, sh_of)
    hi = np.maximum.outer(sh_of, sh_of)
    drop = np.zeros((b.nbf, b.nbf), dtype=bool)
    for a, c in unused:
        drop |= (lo == a) & (hi == c)
    assert drop.sum() > 0
    S, H = b.one_electron()
    eri = b.eri_dense()
    assert np.abs(eri[drop]).max() < 1e-16        # every integral of a dropped row
    nocc = b.nelectrons() // 2
    r = oracle.rhf(S, H, eri, nocc, b.nuclear_repulsion())
    e_full = oracle.rmp2(r["C"], r["eps"], eri, nocc)
    cut = eri.copy()
    cut[drop] = 0.0
    cut[:, :, drop] = 0.0
    e_cut = oracle.rmp2(r["C"], r["eps"], cut, nocc)
    assert abs(e_cut - e_full) < 1e-12, e_cut - e_full
