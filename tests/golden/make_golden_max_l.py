"""Max_L golden values from the upstream pychem reference.

Run once where the reference tree is present, its path in the environment
variable ``PYCHEM_REFERENCE`` (required):

    python tests/golden/make_golden_max_l.py

``Max_L`` drops every shell above that angular momentum (``Util/structures.py:386-390,
815-826``).  Water / cc-pVDZ with Max_L 0 and 1: basis size and RHF energy from the
patched reference, into ``max_l.json``.  The geometry is this project's own.
"""
import json
import math
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import refrun  # noqa: E402


def water():
    th = math.radians(104.52)
    return [["O", 8.0, 0.0, 0.0, 0.0], ["H", 1.0, 0.9572, 0.0, 0.0],
            ["H", 1.0, 0.9572 * math.cos(th), 0.9572 * math.sin(th), 0.0]]


def main():
    root = refrun.prepare()
    ns = refrun.load(root)
    out = {"coords": water(), "basis": "cc-pVDZ", "cases": {}}
    for max_l in (0, 1):
        mol, st = refrun.molecule_from_spec(ns, water(), "cc-pVDZ", extra={"Max_L": max_l})
        ns["hartree_fock"].do(st, mol, st.BasisSets[0], 0)
        out["cases"][str(max_l)] = {"nbf": mol.NOrbitals, "E_hf": float(mol.States[0].TotalEnergy)}
    with open(os.path.join(HERE, "max_l.json"), "w") as fh:
        json.dump(out, fh, indent=1)


if __name__ == "__main__":
    main()
