"""Open-shell golden fixtures (UHF, CUHF, UMP2) from the upstream pychem reference.

Run once where the reference tree is present, its path in the environment
variable ``PYCHEM_REFERENCE`` (required):

    python tests/golden/make_golden_open_shell.py

Each case runs the patched reference (``refrun``: Python-3 patches, regenerated Boys
table, |dE| < 1e-11) through ``hartree_fock.do`` with the given reference type and,
where marked, ``mp2.do``; it writes ``<case>.npz`` with S, core H, the dense ERI
tensor, the electron counts and the final energies.  The reference's own printed
results for ``Tests/example1.inp`` (H3 doublet, CUHF, MP2) go to
``open_shell_energies.json`` next to the tight re-run.  Two MOM cases run the
ground state and the alpha HOMO -> LUMO excited state the way ``pychem.py`` does.
"""
import json
import math
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import refrun  # noqa: E402

H3 = [["H", 1.0, 0.0, 0.0, 0.0], ["H", 1.0, 1.0, 0.0, 0.0], ["H", 1.0, 0.4, 1.0, 0.0]]
OH = [["O", 8.0, 0.0, 0.0, 0.0], ["H", 1.0, 0.97, 0.0, 0.0]]


def water():
    th = math.radians(104.52)
    return [["O", 8.0, 0.0, 0.0, 0.0], ["H", 1.0, 0.9572, 0.0, 0.0],
            ["H", 1.0, 0.9572 * math.cos(th), 0.9572 * math.sin(th), 0.0]]


CASES = [
    # name, coords, basis, charge, multiplicity, reference, mp2
    ("h3_cuhf_sto3g", H3, "STO-3G", 0, 2, "CUHF", True),
    ("h3_uhf_631g", H3, "6-31G", 0, 2, "UHF", True),
    ("oh_uhf_631g", OH, "6-31G", 0, 2, "UHF", True),
    ("oh_cuhf_631g", OH, "6-31G", 0, 2, "CUHF", False),
    ("h2o_cation_uhf_631g", water(), "6-31G", 1, 2, "UHF", False),
]


def run(ns, name, coords, basis, charge, mult, ref, mp2):
    mol, st = refrun.molecule_from_spec(ns, coords, basis, charge=charge, multiplicity=mult, reference=ref,
                                        method="MP2" if mp2 else "HF")
    ns["hartree_fock"].do(st, mol, st.BasisSets[0], 0)
    state = mol.States[0]
    out = dict(basis=np.array(basis), atoms=np.array([a[0] for a in coords]),
               charges=np.array([a[1] for a in coords], dtype=float),
               coords_bohr=np.array([a.Coordinates for a in mol.Atoms], dtype=float),
               charge=np.array(charge), multiplicity=np.array(mult), reference=np.array(ref),
               n_alpha=np.array(mol.NAlphaElectrons), n_beta=np.array(mol.NBetaElectrons),
               S=mol.Overlap.copy(), H=mol.Core.copy(), E_nuc=np.array(mol.NuclearRepulsion),
               eri_dense=mol.CoulombIntegrals.copy(), E_scf=np.array(state.TotalEnergy),
               eps_alpha=np.array(state.Alpha.Energies), eps_beta=np.array(state.Beta.Energies))
    if mp2:
        ecorr = ns["mp2"].do(st, mol)
        ecorr = float(ecorr[0]) if isinstance(ecorr, (list, tuple)) else float(ecorr)
        out["E_mp2_corr"] = np.array(ecorr)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print("%-22s N=%3d  %s E=%.12f%s" % (name, mol.NOrbitals, ref, state.TotalEnergy,
          ("  E_mp2_corr=%.12f" % out["E_mp2_corr"]) if mp2 else ""))
    return out


MOM_CASES = [
    # name, coords, basis: ground state, then the alpha HOMO -> LUMO state by MOM
    ("h2_mom_631g", [["H", 1.0, 0.0, 0.0, 0.0], ["H", 1.0, 0.74, 0.0, 0.0]], "6-31G"),
    ("hf_mom_sto3g", [["F", 9.0, 0.0, 0.0, 0.0], ["H", 1.0, 0.92, 0.0, 0.0]], "STO-3G"),
]


def run_mom(ns, name, coords, basis):
    """pychem.py:64-86 for Excitations = HOMO-LUMO, UHF: the ground state, then the
    excited state's orbitals from the ground state's (structures.reorder_MOs) and an
    SCF with MOM against them (FIXED reference, the default)."""
    coords = water() if coords == "water" else coords
    mol, st = refrun.molecule_from_spec(ns, coords, basis, reference="UHF", extra={"Excitations": "HOMO-LUMO"})
    hf = ns["hartree_fock"]
    hf.do(st, mol, st.BasisSets[0], 0)
    ground, exc = mol.States[0], mol.States[1]
    exc.Alpha.MOs = ns["structures"].reorder_MOs(ground.Alpha.MOs, exc.Alpha.Occupancy)
    exc.Beta.MOs = ns["structures"].reorder_MOs(ground.Beta.MOs, exc.Beta.Occupancy)
    start_a, start_b = exc.Alpha.MOs.copy(), exc.Beta.MOs.copy()
    hf.do(st, mol, st.BasisSets[0], 1, initial_run=False)
    out = dict(basis=np.array(basis), atoms=np.array([a[0] for a in coords]),
               charges=np.array([a[1] for a in coords], dtype=float),
               coords_bohr=np.array([a.Coordinates for a in mol.Atoms], dtype=float),
               charge=np.array(0), multiplicity=np.array(1),
               n_alpha=np.array(mol.NAlphaElectrons), n_beta=np.array(mol.NBetaElectrons),
               S=mol.Overlap.copy(), H=mol.Core.copy(), E_nuc=np.array(mol.NuclearRepulsion),
               eri_dense=mol.CoulombIntegrals.copy(), E_ground=np.array(ground.TotalEnergy),
               E_excited=np.array(exc.TotalEnergy), start_alpha=start_a, start_beta=start_b,
               ground_alpha=ground.Alpha.MOs.copy(), ground_beta=ground.Beta.MOs.copy())
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print("%-22s N=%3d  ground %.12f  HOMO->LUMO (MOM) %.12f" % (name, mol.NOrbitals, ground.TotalEnergy,
                                                                exc.TotalEnergy))
    return out


def printed_example1():
    text = open(os.path.join(refrun.REFERENCE, "Tests", "example1.out")).read()
    hf = re.findall(r"Final HF energy:\s*([-0-9.eE+]+)", text)
    mp2 = re.findall(r"Total MP2 energy:\s*([-0-9.eE+]+)", text)
    return {"printed_final_hf": float(hf[-1]) if hf else None,
            "printed_mp2_corr": float(mp2[-1]) if mp2 else None}


def main():
    root = refrun.prepare()
    ns = refrun.load(root)
    res = {}
    for case in CASES:
        out = run(ns, *case)
        res[case[0]] = {"E_scf": float(out["E_scf"]), "E_mp2_corr": float(out["E_mp2_corr"]) if "E_mp2_corr" in out else None}
    for case in MOM_CASES:
        out = run_mom(ns, *case)
        res[case[0]] = {"E_ground": float(out["E_ground"]), "E_excited": float(out["E_excited"])}
    res["example1_printed"] = printed_example1()
    with open(os.path.join(HERE, "open_shell_energies.json"), "w") as fh:
        json.dump(res, fh, indent=1)


if __name__ == "__main__":
    main()
