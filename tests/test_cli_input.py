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
