"""Multi-basis (bootstrap) golden fixtures from the upstream pychem reference.

Run once where the reference tree is present, its path in the environment
variable ``PYCHEM_REFERENCE`` (required):

    python tests/golden/make_golden_bootstrap.py

Each case runs ``pychem.do_calculation``: the states of its excitation keyword in the
first basis (``pychem.py:62-93``), then for every later basis the orbitals fitted by
``Methods/basis_fit.py`` and the states again (``pychem.py:96-117``).  Every
``hartree_fock.do`` call is wrapped to record (basis, state, final energy, orbitals);
``bootstrap.json`` holds the energies, ``bootstrap.npz`` the orbitals.  The geometries
are this project's own.
"""
import json
import math
import os
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


H2 = [["H", 1.0, 0.0, 0.0, 0.0], ["H", 1.0, 0.74, 0.0, 0.0]]
LIH = [["Li", 3.0, 0.0, 0.0, 0.0], ["H", 1.0, 1.6, 0.0, 0.0]]
CASES = [
    # name, coords, bases, reference, excitations
    ("states_lih_singles_sto3g", LIH, ["STO-3G"], "UHF", "SINGLES"),
    ("states_h2_sd_631g", H2, ["6-31G"], "UHF", "SINGLES-DOUBLES"),
    ("states_lih_sfs_hf_sto3g", LIH, ["STO-3G"], "UHF", "SFS"),
    ("boot_h2_mom_sto3g_631g", H2, ["STO-3G", "6-31G"], "UHF", "HOMO-LUMO"),
    ("boot_h2_mom_sto3g_ccpvdz", H2, ["STO-3G", "cc-pVDZ"], "UHF", "HOMO-LUMO"),
    ("boot_lih_mom_sto3g_631g", LIH, ["STO-3G", "6-31G"], "UHF", "HOMO-LUMO"),
    ("boot_h2o_rhf_sto3g_631g_ccpvdz", water(), ["STO-3G", "6-31G", "cc-pVDZ"], "RHF", None),
    ("boot_lih_mom_constrained_sto3g_631g", LIH, ["STO-3G", "6-31G"], "UHF", "HOMO-LUMO"),
    ("states_h2o_homo_lumo_constrained_sto3g", water(), ["STO-3G"], "UHF", "HOMO-LUMO"),
]
CONSTRAINED = {"boot_lih_mom_constrained_sto3g_631g", "states_h2o_homo_lumo_constrained_sto3g"}


def main():
    root = refrun.prepare()
    ns = refrun.load(root)
    sys.path.insert(0, root)
    import importlib
    cwd = os.getcwd()
    os.chdir(tempfile.mkdtemp(prefix="pychem_boot_"))
    summary, arrays = {}, {}
    try:
        pychem = importlib.import_module("pychem")
        hf = sys.modules["Methods.hartree_fock"]
        do = hf.do
        for name, coords, bases, ref, exc in CASES:
            calls = []

            def wrapped(settings, molecule, basis_set, index, initial_run=True):
                out = do(settings, molecule, basis_set, index, initial_run=initial_run)
                s = molecule.States[index]
                calls.append((basis_set, index, float(s.TotalEnergy), s.Alpha.MOs.copy(), s.Beta.MOs.copy()))
                return out

            hf.do = wrapped
            pychem.hartree_fock.do = wrapped
            extra = {"Max_SCF_Iterations": 300}
            if exc:
                extra["Excitations"] = exc
            if name in CONSTRAINED:
                extra["Constrain_Excited"] = True
            mol, st = refrun.molecule_from_spec(ns, coords, bases[0], reference=ref, extra=extra)
            st.BasisSets = [b.replace("-", "").upper() for b in bases]
            st.OutFileName = name + ".out"
            pychem.do_calculation(st, mol)
            hf.do = do
            pychem.hartree_fock.do = do
            summary[name] = {"bases": bases, "reference": ref, "excitations": exc, "coords": coords,
                             "constrain_excited": name in CONSTRAINED,
                             "calls": [[c[0], c[1], c[2]] for c in calls]}
            for k, c in enumerate(calls):
                arrays["%s_%d_alpha" % (name, k)] = c[3]
                arrays["%s_%d_beta" % (name, k)] = c[4]
            print("%-32s %s" % (name, [(c[0], c[1], round(c[2], 8)) for c in calls]))
    finally:
        os.chdir(cwd)
    with open(os.path.join(HERE, "bootstrap.json"), "w") as fh:
        json.dump(summary, fh, indent=1)
    np.savez_compressed(os.path.join(HERE, "bootstrap.npz"), **arrays)


if __name__ == "__main__":
    main()
