"""Electron-scattering intensities on CPU: the oracle's j0(S r12) integrals and
intensities against the reference's fixtures, and its restatement of the reference's
spherical Bessel scheme.

Fixtures: tests/golden/scat_*.npz from make_golden_scattering.py.  ``clean`` are the
reference's intensities from integrals evaluated into a zeroed tensor; ``printed`` is
its own output table, which differs where its Schwarz screen drops quartets (those keep
the previous pass's values in the reference's integral tensor).
"""
import glob
import math
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


def _reference_form_fundamentals(sP, UP, P, sQ, UQ, Q, lmax, S):
    """two_electron_scattering.c:6-81 restated with the oracle's Bessel scheme:
    U_P U_Q exp(-S^2 (sigma_P + sigma_Q)/4) S^2m z^-m j_m(z), z = S |P - Q|."""
    nbra, nket = sP.size, sQ.size
    out = np.zeros((lmax + 1, nbra, nket))
    Pf, Qf = P.reshape(nbra, 3), Q.reshape(nket, 3)
    for i in range(nbra):
        for k in range(nket):
            U = UP.flat[i] * UQ.flat[k]
            r2 = float(np.sum((Pf[i] - Qf[k]) ** 2))
            if S < 1e-14:
                out[0, i, k] = U
                continue
            eS = math.exp(-0.25 * S * S * (sP.flat[i] + sQ.flat[k]))
            s2 = np.array([S ** (2 * m) for m in range(lmax + 1)])
            if r2 < 1e-14:
                j = np.array([1.0 / np.prod(np.arange(1, 2 * m + 2, 2)) for m in range(lmax + 1)])
            else:
                j = oracle.sph_bessel_scaled(lmax, S * math.sqrt(r2))
            out[:, i, k] = U * eS * s2 * j
    return out


def test_recorded_scattering_fundamentals():
    """The reference's compiled j0(S r12) fundamentals (recorded by
    make_golden_c_ints_scattering.py) against the restatement, every regime."""
    import json
    with open(os.path.join(HERE, "golden", "c_ints_scattering_calls.json")) as fh:
        manifest = json.load(fh)
    arrays = np.load(os.path.join(HERE, "golden", "c_ints_scattering_calls.npz"))
    n = 0
    for call in manifest:
        if call["fn"] != "two_electron_fundamentals":
            continue
        a = call["args"]
        get = lambda k: arrays[a[k][1]]
        lmax, itype, S = int(a[12][1]), int(a[13][1]), float(a[14][1])
        assert itype == 1
        want = arrays[[o for i, o in call["outputs"] if i == 0][0]]
        got = _reference_form_fundamentals(get(1), get(2), get(3), get(4), get(5), get(6), lmax, S)
        scale = max(1.0, float(np.abs(want).max()))
        assert np.abs(got.reshape(want.shape) - want).max() <= 1e-13 * scale, S
        n += 1
    assert n == 24
