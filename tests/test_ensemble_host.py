"""Host-side planning of the ensemble engine (no GPU): the per-atom table."""
import numpy as np
import pytest

from pychem_gb300.ensemble import atom_table


def test_atom_table_offsets():
    from pychem_gb300 import workloads as W
    from pychem_gb300.molecule import Molecule
    mols = [Molecule(c, "6-31G") for c in W.ensemble(n=7, seed=3)]
    at = atom_table(mols)
    for m, mol in enumerate(mols):
        rows = np.nonzero(at["mol"] == m)[0]
        assert rows[0] == at["atom0"][m] and len(rows) == at["nat"][m] == mol.NAtom
        ao = 0
        for r, (sym, Z, xyz) in zip(rows, mol.atoms):
            assert at["ao0"][r] == ao and at["sym"][r] == sym and np.allclose(at["xyz"][r], xyz)
            ao += at["nao"][r]
        assert ao == mol.NOrbitals
