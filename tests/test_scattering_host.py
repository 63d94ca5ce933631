"""Electron-scattering intensities on CPU: the oracle's j0(S r12) integrals and
intensities against the reference's fixtures, and its restatement of the reference's
spherical Bessel scheme.

Fixtures: tests/golden/scat_*.npz from make_golden_scattering.py.  ``clean`` are the
reference's intensities from integrals evaluated into a zeroed tensor; ``printed`` is
its own output table, which differs where its Schwarz screen drops quartets (those keep
the previous pass's values in the reference's integral tensor).
"""
import glob
import os

import numpy as np
import pytest

from oracle import oracle

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = sorted(glob.glob(os.path.join(HERE, "golden", "scat_*.npz")))
NAMES = [os.path.basename(c)[:-4] for c in CASES]


def load(name):
    return np.load(os.path.join(HERE, "golden", name + ".npz"))


def oracle_basis(z):
    atoms = [(str(a), float(c), *x) for a, c, x in zip(z["atoms"], z["charges"], z["coords_bohr"])]
    return oracle.Basis(atoms, str(z["basis"]))


def test_fixtures_present():
    assert len(CASES) >= 5


@pytest.mark.parametrize("name", NAMES)
def test_oracle_scattering_integrals(name):
    z = load(name)
    b = oracle_basis(z)
    for k, gi in enumerate(z["eri_index"]):
        eri = b.eri_dense(scattering=float(z["grid"][gi]))
        assert np.abs(eri - z["eri_clean"][k]).max() < 1e-13, float(z["grid"][gi])


@pytest.mark.parametrize("name", [n for n in NAMES if "ccpvdz" not in n])
def test_oracle_intensities(name):
    z = load(name)
    b = oracle_basis(z)
    for gi, S in enumerate(z["grid"]):
        eri = b.eri_dense(scattering=float(S))
        for st in range(len(z["density_alpha"])):
            I = oracle.scattering_intensity(z["density_alpha"][st], z["density_beta"][st], eri,
                                            int(z["n_electrons"]))
            assert abs(I - z["clean"][gi][st]) < 1e-10


@pytest.mark.parametrize("name", [n for n in NAMES if "ccpvdz" not in n])
def test_printed_table_equals_clean_without_screening(name):
    """Where the scattering Schwarz screen keeps every quartet the reference's printed
    table equals the clean intensities; differences only appear at grid values where it
    drops some (S = 0 on separated pairs, large S)."""
    z = load(name)
    b = oracle_basis(z)
    n_all = b.nshell * (b.nshell + 1) // 2
    n_all = n_all * (n_all + 1) // 2
    for gi, S in enumerate(z["grid"]):
        oracle.lib().oracle_set_operator(1, float(S))
        try:
            kept = len(b.quartets())
        finally:
            oracle.lib().oracle_set_operator(0, 0.0)
        diff = np.abs(z["printed"][gi] - z["clean"][gi]).max()
        if kept == n_all:
            assert diff < 1e-9, (float(S), diff)
        elif diff > 1e-9:
            assert kept < n_all


def test_bessel_regimes():
    """The restated scheme against scipy's spherical Bessel functions: series and
    recursion to 1e-12 (5e-12 just below z = 10, where the reference's 20-term series
    cancels), the two-term asymptotic form to its own truncation error."""
    sp = pytest.importorskip("scipy.special")
    for z in (1e-4, 0.05, 0.7, 3.0, 9.5, 10.5, 42.0, 99.0):
        got = oracle.sph_bessel_scaled(8, z)
        ref = np.array([sp.spherical_jn(m, z) / z ** m for m in range(9)])
        assert np.abs(got - ref).max() < (5e-12 if 5.0 < z < 10.0 else 1e-12), z
    for z in (150.0, 1000.0):
        got = oracle.sph_bessel_scaled(4, z)
        ref = np.array([sp.spherical_jn(m, z) / z ** m for m in range(5)])
        assert np.all(np.abs(got - ref) <= 10.0 / z ** 2 * np.abs(ref).max() + 1e-18), z
    assert np.array_equal(oracle.sph_bessel_scaled(3, 0.0), [1.0, 1.0 / 3, 1.0 / 15, 1.0 / 105])


def test_zero_momentum_transfer_gives_n_squared():
    """At S = 0 the integrals are S_ab S_cd and I = N^2 for any idempotent state."""
    z = load("scat_lih_uhf_631g")
    n = int(z["n_electrons"])
    assert abs(z["clean"][0][0] - n * n) < 1e-9
