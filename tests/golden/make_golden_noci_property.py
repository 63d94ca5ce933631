"""NOCI followed by scattering properties, from the upstream pychem reference.

Run once where the reference tree is present, its path in the environment
variable ``PYCHEM_REFERENCE`` (required):

    python tests/golden/make_golden_noci_property.py

H2 (0.9 A, 6-31G), Method NOCI over the ground and HOMO -> LUMO states, Job_Type
PROPERTY with the scattering intensities on two grid values: upstream evaluates the
properties over ``molecule.States`` after ``noci.do`` (``pychem.py:126-134``), one
column per state.  (With a spin-flip list upstream's property step fails: its table
is sized by the Hartree-Fock state count while ``molecule.States`` holds the
determinants, ``properties.py:13-23``.)  ``noci_property.json`` holds the NOCI energies and the printed table
(grid values where the scattering screen drops no quartet, so the printed values are
the clean ones).  The geometry is this project's own.
"""
import json
import os
import re
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import refrun  # noqa: E402

COORDS = [["H", 1.0, 0.0, 0.0, 0.0], ["H", 1.0, 0.9, 0.0, 0.0]]
GRID = [0.5, 1.0]


def main():
    root = refrun.prepare()
    ns = refrun.load(root)
    sys.path.insert(0, root)
    import importlib
    cwd = os.getcwd()
    os.chdir(tempfile.mkdtemp(prefix="pychem_nociprop_"))
    try:
        pychem = importlib.import_module("pychem")
        mol, st = refrun.molecule_from_spec(ns, COORDS, "6-31G", reference="UHF", method="NOCI",
                                            extra={"Excitations": "HOMO-LUMO", "Constrain_Excited": True,
                                                   "Max_SCF_Iterations": 300, "Job_Type": "PROPERTY",
                                                   "Property_Type": "SCATTERING", "Property_Grid": GRID})
        st.OutFileName = "h2.out"
        pychem.do_calculation(st, mol)
        text = open("h2.out").read()
        i = text.index("Scattering patterns for each electronic state")
        rows = []
        for line in text[i:].splitlines()[1:]:
            nums = re.findall(r"[-+]?\d+\.\d+(?:[eE][-+]?\d+)?", line)
            if len(nums) == len(mol.States) + 1:
                rows.append([float(x) for x in nums[1:]])
            elif rows:
                break
    finally:
        os.chdir(cwd)
    out = {"coords": COORDS, "basis": "6-31G", "excitations": "HOMO-LUMO", "grid": GRID,
           "noci_energies": [float(e) for e in mol.NOCIEnergies], "intensities": rows}
    with open(os.path.join(HERE, "noci_property.json"), "w") as fh:
        json.dump(out, fh, indent=1)
    print(out)


if __name__ == "__main__":
    main()
