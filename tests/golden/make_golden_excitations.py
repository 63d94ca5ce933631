"""State and spin-flip determinant lists from the upstream pychem reference.

Run once where the reference tree is present, its path in the environment
variable ``PYCHEM_REFERENCE`` (required):

    python tests/golden/make_golden_excitations.py

For each molecule and each excitation keyword (or custom excitation lists) the
patched reference builds its Molecule (``Util/structures.py:process_input``, which
calls ``set_excitations``, ``structures.py:526-657``); the occupancy lists of
``molecule.States``, ``molecule.SpinFlipStates`` and the core-orbital count go to
``excitation_lists.json``; inputs that the reference rejects (custom excitation lists:
``set_excitations`` has no branch for them and exits) are recorded as rejected.  No SCF
runs.  The geometries are this project's own.
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


MOLECULES = [
    # name, coords, basis, charge, multiplicity
    ("LiH", [["Li", 3.0, 0.0, 0.0, 0.0], ["H", 1.0, 1.6, 0.0, 0.0]], "6-31G", 0, 1),
    ("H2O", water(), "STO-3G", 0, 1),
    ("OH", [["O", 8.0, 0.0, 0.0, 0.0], ["H", 1.0, 0.97, 0.0, 0.0]], "6-31G", 0, 2),
    ("C2", [["C", 6.0, 0.0, 0.0, 0.0], ["C", 6.0, 1.25, 0.0, 0.0]], "6-31G", 0, 1),
]
KEYWORDS = ["HOMO-LUMO", "SINGLES", "DOUBLES", "SINGLES-DOUBLES", "DOUBLE-PAIRED", "SFS", "SFD", "SFSD",
            "SF-S", "SPIN-FLIP-DOUBLES", "SFS-CISD", "SFD-CISD", "SFD-CISDT", "SFD-CISDTQ", "SFSD-CISD",
            "SFSD-CISDT", "SFSD-CISDTQ"]
CUSTOM = [
    # (Alpha_Excitations, Beta_Excitations); None leaves the key out
    ([[1, 5], [0, 6]], None),
    (None, [[1, 4]]),
    ([[1, 5], []], [[], [0, 4]]),
]


def main():
    root = refrun.prepare()
    ns = refrun.load(root)
    out = []
    for name, coords, basis, charge, mult in MOLECULES:
        cases = [({"Excitations": k}, k, None, None) for k in KEYWORDS
                 if not (name == "C2" and k in ("DOUBLES", "SINGLES-DOUBLES"))]
        for a, b in CUSTOM:
            extra = {}
            if a is not None:
                extra["Alpha_Excitations"] = a
            if b is not None:
                extra["Beta_Excitations"] = b
            cases.append((extra, None, a, b))
        for extra, kw, a, b in cases:
            try:
                mol, st = refrun.molecule_from_spec(ns, coords, basis, charge=charge, multiplicity=mult,
                                                    reference="UHF", extra=extra)
            except SystemExit:
                # custom excitation lists stop the reference in set_excitations
                out.append({"molecule": name, "alpha_excitations": a, "beta_excitations": b,
                            "excitations": kw, "rejected": True})
                continue
            out.append({"molecule": name, "basis": basis, "charge": charge, "multiplicity": mult,
                        "n_alpha": mol.NAlphaElectrons, "n_beta": mol.NBetaElectrons, "n_orbitals": mol.NOrbitals,
                        "n_core": mol.NCoreOrbitals, "charges": [a_[1] for a_ in coords],
                        "excitations": kw, "alpha_excitations": a, "beta_excitations": b,
                        "states": [[list(map(int, s.Alpha.Occupancy)), list(map(int, s.Beta.Occupancy))]
                                   for s in mol.States],
                        "spin_flip": [[int(x[0]), list(map(int, x[1])), list(map(int, x[2]))]
                                      for x in mol.SpinFlipStates]})
            print("%-4s %-14s states=%3d spin-flip=%3d" % (name, kw or "custom %s/%s" % (a, b), len(out[-1]["states"]),
                                                          len(out[-1]["spin_flip"])))
    with open(os.path.join(HERE, "excitation_lists.json"), "w") as fh:
        json.dump(out, fh)


if __name__ == "__main__":
    main()
