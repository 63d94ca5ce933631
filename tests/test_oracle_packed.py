"""The oracle's packed-store path (oracle.PackedStore, rhf(store=...), rmp2_packed)
against its dense-tensor path, which the golden fixtures pin to the reference.  The
packed path carries the energies of the two large benchmark configurations
(tests/golden/configs.json), where no dense tensor fits; here it must reproduce the
dense path on a jittered water dimer (6-31G) and on water in cc-pVDZ (d shells):
blocks, Coulomb and exchange matrices for non-symmetric densities, RHF and MP2."""
import math
import os

import numpy as np
import pytest

from oracle import oracle as O


def _dimer(golden_dir):
    g = np.load(os.path.join(golden_dir, "water_dimer_631g.npz"))
    atoms = [(str(s), float(z), *map(float, xyz)) for s, z, xyz in zip(g["atoms"], g["charges"], g["coords_bohr"])]
    return O.Basis(atoms, "6-31G")


def _water_ccpvdz():
    th = math.radians(104.52)
    r = 0.9572 * O.TO_BOHR
    return O.Basis([("O", 8.0, 0.0, 0.0, 0.0), ("H", 1.0, r, 0.0, 0.0),
                    ("H", 1.0, r * math.cos(th), r * math.sin(th), 0.0)], "cc-pVDZ")


@pytest.mark.parametrize("which", ["dimer_631g", "water_ccpvdz"])
def test_packed_store_matches_dense(golden_dir, which):
    b = _dimer(golden_dir) if which == "dimer_631g" else _water_ccpvdz()
    eri = b.eri_dense()
    st = O.PackedStore(b, nthreads=4)
    assert np.array_equal(np.array(b.quartets(), dtype=np.int32), st.quads)
    rng = np.random.default_rng(3)
    Dj = rng.normal(size=(b.nbf, b.nbf))
    Dj = Dj + Dj.T
    Dk = rng.normal(size=(b.nbf, b.nbf))       # exchange with a non-symmetric density
    J, K = st.jk(Dj, Dk)
    np.testing.assert_allclose(J, np.einsum("cd,abcd->ab", Dj, eri), rtol=0, atol=1e-12)
    np.testing.assert_allclose(K, np.einsum("cb,abcd->ad", Dk, eri), rtol=0, atol=1e-12)
    S, H = b.one_electron()
    nocc = b.nelectrons() // 2
    rd = O.rhf(S, H, eri, nocc, b.nuclear_repulsion())
    rp = O.rhf(S, H, None, nocc, b.nuclear_repulsion(), store=st)
    assert rd["converged"] and rp["converged"]
    assert abs(rd["E"] - rp["E"]) < 1e-10
    e_dense = O.rmp2(rd["C"], rd["eps"], eri, nocc)
    e_packed = O.rmp2_packed(rd["C"], rd["eps"], st, nocc)
    assert abs(e_dense - e_packed) < 1e-12


def test_config_fixtures_present(golden_dir):
    import json
    d = json.load(open(os.path.join(golden_dir, "configs.json")))
    c2, c3 = d["c2_water16_631g"], d["c3_c12h26_ccpvdz"]
    assert (c2["nbf"], c2["nocc"], c3["nbf"], c3["nocc"]) == (208, 80, 298, 49)
    assert c2["converged"] and c3["converged"]
