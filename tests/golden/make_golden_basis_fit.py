"""Basis-fitting golden fixtures from the upstream pychem reference.

Run once where the reference tree is present, its path in the environment
variable ``PYCHEM_REFERENCE`` (required):

    python tests/golden/make_golden_basis_fit.py

For each case the patched reference builds the molecule in the old basis and projects
a seeded random square MO matrix into the new basis with ``Methods/basis_fit.py:6-21``
(the fit is linear in the MO coefficients, so random matrices exercise every
function); ``basis_fit.npz`` holds the inputs and the reference's outputs.  The
geometries are this project's own.
"""
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import refrun  # noqa: E402


def water():
    th = math.radians(104.52)
    return [["O", 8.0, 0.0, 0.0, 0.0], ["H", 1.0, 0.9572, 0.0, 0.0],
            ["H", 1.0, 0.9572 * math.cos(th), 0.9572 * math.sin(th), 0.0]]


CASES = [
    # name, coords, old basis, new basis
    ("h2o_sto3g_to_631g", water(), "STO-3G", "6-31G"),
    ("h2o_sto3g_to_ccpvdz", water(), "STO-3G", "cc-pVDZ"),
    ("lih_sto3g_to_631g", [["Li", 3.0, 0.0, 0.0, 0.0], ["H", 1.0, 1.6, 0.0, 0.0]], "STO-3G", "6-31G"),
    ("c2_sto3g_to_ccpvdz", [["C", 6.0, 0.0, 0.0, 0.0], ["C", 6.0, 1.25, 0.0, 0.0]], "STO-3G", "cc-pVDZ"),
    ("h2_631g_to_ccpvdz", [["H", 1.0, 0.0, 0.0, 0.0], ["H", 1.0, 0.74, 0.0, 0.0]], "6-31G", "cc-pVDZ"),
]


def main():
    root = refrun.prepare()
    ns = refrun.load(root)
    sys.path.insert(0, os.path.join(root, "Methods"))
    import basis_fit
    rng = np.random.default_rng(11)
    out = {}
    for name, coords, old, new in CASES:
        mol, st = refrun.molecule_from_spec(ns, coords, old)
        n = mol.NOrbitals
        C = rng.standard_normal((n, n))
        new_clean = new.replace("-", "").upper()
        fitted = basis_fit.do(mol, C.copy(), new_clean)
        out[name + "_C"] = C
        out[name + "_fitted"] = np.array(fitted, dtype=float)
        out[name + "_meta"] = np.array([old, new])
        out[name + "_coords"] = np.array([[a[1], *a[2:]] for a in coords], dtype=float)
        out[name + "_atoms"] = np.array([a[0] for a in coords])
        print("%-22s %3d -> %s" % (name, n, np.array(fitted).shape))
    np.savez_compressed(os.path.join(HERE, "basis_fit.npz"), **out)


if __name__ == "__main__":
    main()
