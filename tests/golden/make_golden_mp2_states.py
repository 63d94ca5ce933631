"""MP2 over ground and excited states from the upstream pychem reference.

Run once where the reference tree is present, its path in the environment
variable ``PYCHEM_REFERENCE`` (required):

    python tests/golden/make_golden_mp2_states.py

``Method = "MP2"`` with ``Excitations = "HOMO-LUMO"``: upstream converges the ground
and the MOM excited state, then ``mp2.do`` evaluates MP2 for every state with that
state's own orbitals and orbital energies (``Methods/mp2.py:16-121``).  The printed
per-state total MP2 energies and the state energies go to ``mp2_states.json``, the
states' final orbitals to ``mp2_states.npz``.  The geometries are this project's own.
"""
import json
import math
import os
import re
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import refrun  # noqa: E402


def water():
    th = math.radians(104.52)
    return [["O", 8.0, 0.0, 0.0, 0.0], ["H", 1.0, 0.9572, 0.0, 0.0],
            ["H", 1.0, 0.9572 * math.cos(th), 0.9572 * math.sin(th), 0.0]]


CASES = [
    ("h2_mp2_states_631g", [["H", 1.0, 0.0, 0.0, 0.0], ["H", 1.0, 0.74, 0.0, 0.0]], "6-31G", "UHF"),
    ("h2o_mp2_states_sto3g_cuhf", water(), "STO-3G", "CUHF"),
]


def main():
    root = refrun.prepare()
    ns = refrun.load(root)
    sys.path.insert(0, root)
    import importlib
    cwd = os.getcwd()
    os.chdir(tempfile.mkdtemp(prefix="pychem_mp2states_"))
    out, orbitals = {}, {}
    try:
        pychem = importlib.import_module("pychem")
        for name, coords, basis, ref in CASES:
            mol, st = refrun.molecule_from_spec(ns, coords, basis, reference=ref, method="MP2",
                                                extra={"Excitations": "HOMO-LUMO", "Max_SCF_Iterations": 300})
            st.OutFileName = name + ".out"
            pychem.do_calculation(st, mol)
            text = open(name + ".out").read()
            mp2 = [float(x) for x in re.findall(r"Total MP2 energy:\s*([-0-9.eE+]+)", text)]
            out[name] = {"coords": coords, "basis": basis, "reference": ref,
                         "E_hf": [float(s.TotalEnergy) for s in mol.States], "E_mp2_total": mp2}
            for k, s in enumerate(mol.States):
                orbitals["%s_%d_alpha" % (name, k)] = s.Alpha.MOs
                orbitals["%s_%d_beta" % (name, k)] = s.Beta.MOs
            print(name, out[name]["E_hf"], mp2)
    finally:
        os.chdir(cwd)
    with open(os.path.join(HERE, "mp2_states.json"), "w") as fh:
        json.dump(out, fh, indent=1)
    np.savez_compressed(os.path.join(HERE, "mp2_states.npz"), **orbitals)


if __name__ == "__main__":
    main()
