"""NOCI golden fixtures from the upstream pychem reference.

Run once where the reference tree is present, its path in the environment
variable ``PYCHEM_REFERENCE`` (required):

    python tests/golden/make_golden_noci.py

Each case runs the patched reference (``refrun``: Python-3 patches, regenerated Boys
table, |dE| < 1e-11) through ``pychem.do_calculation`` with ``Method = "NOCI"``: the
Hartree-Fock states in the reference's order (high spin first for spin-flip
excitations, ``pychem.py:62-93``), then ``Methods/noci.py:51-122``.  The CI matrix
and overlap are captured at the generalised eigensolver call.  ``<case>.npz`` holds
S, core H, the dense ERI tensor, the Hartree-Fock states (occupancies, orbitals,
energies) before the spin-flip rearrangement, the spin-flip state list of
``Util/structures.py:526-620``, the NOCI determinants' orbitals after it, the CI
matrix, overlap, energies and vectors.  The geometries are this project's own.
"""
import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import refrun  # noqa: E402


def lih(r):
    return [["Li", 3.0, 0.0, 0.0, 0.0], ["H", 1.0, r, 0.0, 0.0]]


def h2(r):
    return [["H", 1.0, 0.0, 0.0, 0.0], ["H", 1.0, r, 0.0, 0.0]]


CASES = [
    # name, coords, basis, excitations
    ("noci_lih_sfs_sto3g", lih(1.9), "STO-3G", "SFS"),
    ("noci_lih_sfs_631g", lih(1.7), "6-31G", "SFS"),
    ("noci_h2_sfs_631g", h2(1.4), "6-31G", "SFS"),
    ("noci_lih_sfs_cisd_sto3g", lih(1.9), "STO-3G", "SFS-CISD"),
    ("noci_lih_sfd_cisd_sto3g", lih(2.1), "STO-3G", "SFD-CISD"),
    ("noci_lih_sfsd_cisd_sto3g", lih(1.9), "STO-3G", "SFSD-CISD"),
    ("noci_h2_homo_lumo_631g", h2(0.9), "6-31G", "HOMO-LUMO"),
    ("noci_c2_sfd_cisd_631g", [["C", 6.0, 0.0, 0.0, 0.0], ["C", 6.0, 1.25, 0.0, 0.0]], "6-31G", "SFD-CISD"),
]


def main():
    root = refrun.prepare()
    ns = refrun.load(root)
    sys.path.insert(0, root)
    import importlib
    cwd = os.getcwd()
    os.chdir(tempfile.mkdtemp(prefix="pychem_noci_"))
    try:
        pychem = importlib.import_module("pychem")
        noci = sys.modules["Methods.noci"]
        captured = {}
        gen_eig = noci.gen_eig
        reorder = noci.reorder_orbitals

        def eig_capture(H, S):
            captured["H"], captured["S"] = H.copy(), S.copy()
            return gen_eig(H, S)

        def reorder_capture(molecule):
            captured["hf_states"] = [(list(s.Alpha.Occupancy), list(s.Beta.Occupancy), s.Alpha.MOs.copy(),
                                      s.Beta.MOs.copy(), float(s.TotalEnergy)) for s in molecule.States]
            return reorder(molecule)

        noci.gen_eig = eig_capture
        noci.reorder_orbitals = reorder_capture
        summary = {}
        for name, coords, basis, exc in CASES:
            captured.clear()
            mol, st = refrun.molecule_from_spec(ns, coords, basis, reference="UHF", method="NOCI",
                                                extra={"Excitations": exc, "Constrain_Excited": True,
                                                       "Max_SCF_Iterations": 300})
            st.OutFileName = name + ".out"
            pychem.do_calculation(st, mol)
            hf = captured.get("hf_states") or [(list(s.Alpha.Occupancy), list(s.Beta.Occupancy), s.Alpha.MOs.copy(),
                                                 s.Beta.MOs.copy(), float(s.TotalEnergy)) for s in mol.States]
            sf = mol.SpinFlipStates
            out = dict(basis=np.array(basis), excitations=np.array(exc), reference=np.array("UHF"),
                       constrain_excited=np.array(True),
                       atoms=np.array([a[0] for a in coords]),
                       charges=np.array([a[1] for a in coords], dtype=float),
                       coords_bohr=np.array([a.Coordinates for a in mol.Atoms], dtype=float),
                       n_alpha=np.array(mol.NAlphaElectrons), n_beta=np.array(mol.NBetaElectrons),
                       S=mol.Overlap.copy(), H=mol.Core.copy(), E_nuc=np.array(mol.NuclearRepulsion),
                       eri_dense=mol.CoulombIntegrals.copy(),
                       hf_occ_alpha=np.array([h[0] for h in hf]), hf_occ_beta=np.array([h[1] for h in hf]),
                       hf_alpha=np.array([h[2] for h in hf]), hf_beta=np.array([h[3] for h in hf]),
                       hf_energies=np.array([h[4] for h in hf]),
                       sf_index=np.array([s[0] for s in sf], dtype=int),
                       sf_alpha=np.array([s[1] for s in sf], dtype=int).reshape(len(sf), mol.NOrbitals),
                       sf_beta=np.array([s[2] for s in sf], dtype=int).reshape(len(sf), mol.NOrbitals),
                       det_alpha=np.array([s.Alpha.MOs for s in mol.States]),
                       det_beta=np.array([s.Beta.MOs for s in mol.States]),
                       ci_H=captured["H"], ci_S=captured["S"],
                       noci_energies=np.array(mol.NOCIEnergies), noci_vectors=np.array(mol.NOCIWavefunction))
            np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
            summary[name] = {"excitations": exc, "basis": basis, "hf_energies": [h[4] for h in hf],
                             "noci_energies": [float(e) for e in mol.NOCIEnergies]}
            print("%-26s N=%2d  %-10s dets=%2d  NOCI %s" % (name, mol.NOrbitals, exc, len(mol.States),
                                                          np.array2string(np.array(mol.NOCIEnergies)[:4],
                                                                          precision=8)))
    finally:
        os.chdir(cwd)
    with open(os.path.join(HERE, "noci_energies.json"), "w") as fh:
        json.dump(summary, fh, indent=1)


if __name__ == "__main__":
    main()
