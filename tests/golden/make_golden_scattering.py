"""Electron-scattering golden fixtures from the upstream pychem reference.

Run once where the reference tree is present, its path in the environment
variable ``PYCHEM_REFERENCE`` (required):

    python tests/golden/make_golden_scattering.py

Each case runs the patched reference (``refrun``) through ``pychem.do_calculation``
with ``Job_Type = "PROPERTY"``, ``Property_Type = "SCATTERING"``: the Hartree-Fock
state(s), then ``Methods/properties.py:6-37``, whose table of total scattering
intensities (one column per state) is read back from the output file.  The reference
overwrites ``molecule.CoulombIntegrals`` only for the quartets its scattering Schwarz
screen keeps (``hartree_fock.py:241-327``), so screened-out quartets keep the values of
the previous pass; the generator therefore also evaluates the scattering integrals at
every grid value on a zeroed tensor (``clean``) and stores those tensors and the
intensities they give.  ``<case>.npz`` holds S, the state densities, the grid, the
printed and clean intensities and the clean integral tensors (at the grid indices
``eri_index``).  The geometries are this
project's own.
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


GRID = [0.0, 0.25, 0.5, 1.0, 2.0, 3.5, 6.0]
ALL = list(range(len(GRID)))
CASES = [
    # name, coords, basis, reference, multiplicity, excitations, grid indices whose tensors are kept
    ("scat_h2o_rhf_sto3g", water(), "STO-3G", "RHF", 1, None, ALL),
    ("scat_h2o_rhf_ccpvdz", water(), "cc-pVDZ", "RHF", 1, None, [2, 4]),
    ("scat_lih_uhf_631g", [["Li", 3.0, 0.0, 0.0, 0.0], ["H", 1.0, 1.6, 0.0, 0.0]], "6-31G", "UHF", 1, None, ALL),
    ("scat_h2_mom_631g", [["H", 1.0, 0.0, 0.0, 0.0], ["H", 1.0, 0.74, 0.0, 0.0]], "6-31G", "UHF", 1, "HOMO-LUMO",
     ALL),
    ("scat_oh_uhf_631g", [["O", 8.0, 0.0, 0.0, 0.0], ["H", 1.0, 0.97, 0.0, 0.0]], "6-31G", "UHF", 2, None, ALL),
]


def read_table(path, nstates):
    text = open(path).read()
    i = text.index("Scattering patterns for each electronic state")
    rows = []
    for line in text[i:].splitlines()[1:]:
        nums = re.findall(r"[-+]?\d+\.\d+(?:[eE][-+]?\d+)?", line)
        if len(nums) == nstates + 1:
            rows.append([float(x) for x in nums])
        elif rows:
            break
    return np.array(rows)


def main():
    root = refrun.prepare()
    ns = refrun.load(root)
    sys.path.insert(0, root)
    import importlib
    cwd = os.getcwd()
    os.chdir(tempfile.mkdtemp(prefix="pychem_scat_"))
    summary = {}
    try:
        pychem = importlib.import_module("pychem")
        hf = ns["hartree_fock"]
        for name, coords, basis, ref, mult, exc, keep in CASES:
            extra = {"Job_Type": "PROPERTY", "Property_Type": "SCATTERING", "Property_Grid": GRID,
                     "Max_SCF_Iterations": 300}
            if exc:
                extra["Excitations"] = exc
            mol, st = refrun.molecule_from_spec(ns, coords, basis, reference=ref, multiplicity=mult, method="HF",
                                                extra=extra)
            st.OutFileName = name + ".out"
            pychem.do_calculation(st, mol)
            nst = len(mol.States)
            printed = read_table(name + ".out", nst)
            Da = np.array([s.Alpha.Density for s in mol.States])
            Db = np.array([s.Beta.Density for s in mol.States])
            clean_eri, clean_int = [], []
            for S in GRID:
                mol.CoulombIntegrals[...] = 0.0
                hf.evaluate_2e_ints(mol, 1, S)
                eri = mol.CoulombIntegrals.copy()
                clean_eri.append(eri)
                row = []
                for a, b in zip(Da, Db):
                    t = a + b
                    v = np.einsum("ab,cd,abcd->", t, t, eri) - np.einsum("ad,cb,abcd->", a, a, eri) \
                        - np.einsum("ad,cb,abcd->", b, b, eri)
                    row.append(mol.NElectrons + v)
                clean_int.append(row)
            out = dict(basis=np.array(basis), reference=np.array(ref), multiplicity=np.array(mult),
                       excitations=np.array(exc or ""), atoms=np.array([a[0] for a in coords]),
                       charges=np.array([a[1] for a in coords], dtype=float),
                       coords_bohr=np.array([a.Coordinates for a in mol.Atoms], dtype=float),
                       n_electrons=np.array(mol.NElectrons), S=mol.Overlap.copy(),
                       grid=np.array(GRID), density_alpha=Da, density_beta=Db,
                       state_energies=np.array([s.TotalEnergy for s in mol.States]),
                       printed=printed[:, 1:], clean=np.array(clean_int), eri_index=np.array(keep),
                       eri_clean=np.array([clean_eri[k] for k in keep]))
            np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
            diff = np.abs(printed[:, 1:] - np.array(clean_int)).max()
            summary[name] = {"states": nst, "grid": GRID, "printed": printed[:, 1:].tolist(),
                             "clean": np.array(clean_int).tolist(), "max_printed_minus_clean": float(diff)}
            print("%-22s N=%3d states=%d  I(S) %s  |printed-clean| %.2e" % (
                name, mol.NOrbitals, nst, np.array2string(np.array(clean_int)[:, 0], precision=6), diff))
    finally:
        os.chdir(cwd)
    with open(os.path.join(HERE, "scattering_intensities.json"), "w") as fh:
        json.dump(summary, fh, indent=1)


if __name__ == "__main__":
    main()
