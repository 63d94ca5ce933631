"""Spin-component-scaled MP2 golden values from the upstream pychem reference.

Run once where the reference tree is present, its path in the environment
variable ``PYCHEM_REFERENCE`` (required):

    python tests/golden/make_golden_mp2_scaled.py

For each molecule the patched reference runs ``hartree_fock.do`` and then
``mp2.do`` (``Methods/mp2.py:16-121``) with ``Method`` set to MP2, MP2-SCS and
MP2-SOS; the scaling of ``mp2.py:97-107`` runs under Python 3, so SCS uses 1/3 and
6/5 (Python 2 would truncate both).  ``mp2_scaled.json`` holds the three correlation
energies per molecule with the state energy.  The geometries are this project's own.
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


CASES = [
    # name, coords, basis, multiplicity, reference
    ("h2o_rhf_631g", water(), "6-31G", 1, "RHF"),
    ("oh_uhf_631g", [["O", 8.0, 0.0, 0.0, 0.0], ["H", 1.0, 0.97, 0.0, 0.0]], "6-31G", 2, "UHF"),
    ("lih_uhf_sto3g", [["Li", 3.0, 0.0, 0.0, 0.0], ["H", 1.0, 1.6, 0.0, 0.0]], "STO-3G", 1, "UHF"),
]


def main():
    root = refrun.prepare()
    ns = refrun.load(root)
    out = {}
    for name, coords, basis, mult, ref in CASES:
        mol, st = refrun.molecule_from_spec(ns, coords, basis, multiplicity=mult, reference=ref, method="MP2")
        ns["hartree_fock"].do(st, mol, st.BasisSets[0], 0)
        rec = {"coords": coords, "basis": basis, "multiplicity": mult, "reference": ref,
               "E_hf": float(mol.States[0].TotalEnergy)}
        for method in ("MP2", "MP2-SCS", "MP2-SOS"):
            st.Method = method
            rec[method] = float(ns["mp2"].do(st, mol))
        out[name] = rec
        print(name, rec["E_hf"], rec["MP2"], rec["MP2-SCS"], rec["MP2-SOS"])
    with open(os.path.join(HERE, "mp2_scaled.json"), "w") as fh:
        json.dump(out, fh, indent=1)


if __name__ == "__main__":
    main()
