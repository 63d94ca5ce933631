"""Input-file reading of the command-line runner (no GPU)."""
from pychem_gb300.cli import read_sections


def test_read_sections(tmp_path):
    p = tmp_path / "job.inp"
    p.write_text('[h3]\nMethod = "mp2"\nBasis_Sets = ["STO-3G"]\nMultiplicity = 2\nCharge = 0\n'
                 "Coords = [['H', 1.0, 0., 0., 0.], ['H', 1.0, 1.0, 0., 0.]]\nReference = \"cuhf\"\n"
                 '[water]\nCoords_Units = "bohr"\nCoords = [[\'O\', 8.0, 0., 0., 0.]]\n')
    secs = read_sections(str(p))
    assert [s for s, _ in secs] == ["h3", "water"]
    o = secs[0][1]
    assert o["METHOD"] == "MP2" and o["REFERENCE"] == "CUHF" and o["MULTIPLICITY"] == 2
    assert o["BASIS_SETS"] == ["STO-3G"] and o["COORDS"][1][2] == 1.0
    assert secs[1][1]["COORDS_UNITS"] == "BOHR"


def test_max_l_basis_matches_reference():
    """Max_L drops the shells above it (Util/structures.py:815-826): basis size from
    pychem_gb300.molecule.Molecule and the RHF energy in that basis (oracle) against
    the reference (make_golden_max_l.py)."""
    import json
    import os
    from oracle import oracle
    from pychem_gb300.molecule import Molecule
    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "golden", "max_l.json")) as fh:
        ref = json.load(fh)
    for max_l, case in ref["cases"].items():
        mol = Molecule(ref["coords"], ref["basis"], max_l=int(max_l))
        assert mol.NOrbitals == case["nbf"]
        assert max(s[0] for s in mol.shells) <= int(max_l)
        b = oracle.Basis([(a[0], a[1], *a[2]) for a in mol.atoms], ref["basis"], max_l=int(max_l))
        assert b.nbf == case["nbf"]
        S, H = b.one_electron()
        r = oracle.rhf(S, H, b.eri_dense(), mol.NAlphaElectrons, b.nuclear_repulsion())
        assert abs(r["E"] - case["E_hf"]) < 1e-8


def test_unsupported_options_stop_the_section():
    import pytest
    from pychem_gb300.cli import _check_options
    for opts in ({"CARTESIAN_L": [2]}, {"MOM_REFERENCE": "MUTABLE"}, {"USE_MOM": False, "EXCITATIONS": "HOMO-LUMO"}):
        with pytest.raises(ValueError):
            _check_options(opts)
    _check_options({"CARTESIAN_L": [], "MOM_REFERENCE": "FIXED", "USE_MOM": True})
