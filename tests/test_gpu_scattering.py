"""Electron-scattering intensities on the GPU against the reference fixtures.

* the j0(S r12) integral store (pcg_scattering_class, its own Schwarz screen) against
  the reference's integral tensors at the stored grid values;
* intensities from the reference's state densities against its clean intensities;
* the whole input-file path (SCF on the GPU, then the property table) against them.
"""
import numpy as np
import pytest
import torch

from pychem_gb300 import cli, scattering
from pychem_gb300.engine import GpuEngine
from pychem_gb300.molecule import Molecule

from test_scattering_host import NAMES, load

pytestmark = pytest.mark.gpu


def molecule_for(z):
    coords = [[str(a), float(c), *map(float, x)] for a, c, x in zip(z["atoms"], z["charges"], z["coords_bohr"])]
    return Molecule(coords, str(z["basis"]), multiplicity=int(z["multiplicity"]), units="BOHR"), coords


@pytest.mark.parametrize("name", NAMES)
def test_scattering_integrals(name):
    z = load(name)
    mol, _ = molecule_for(z)
    eng = GpuEngine(mol)
    eng.one_electron()
    for k, gi in enumerate(z["eri_index"]):
        eng.scattering = float(z["grid"][gi])
        eng.schwarz()
        eng.build_tasks()
        eng.compute_eris()
        eri = eng.dense_eri().cpu().numpy()
        assert np.abs(eri - z["eri_clean"][k]).max() < 1e-12, float(z["grid"][gi])


@pytest.mark.parametrize("name", NAMES)
def test_intensities_from_reference_densities(name):
    z = load(name)
    mol, _ = molecule_for(z)
    dens = list(zip(z["density_alpha"], z["density_beta"]))
    table = scattering.intensities(mol, [float(s) for s in z["grid"]], dens)
    assert table.shape == z["clean"].shape
    assert np.abs(table - z["clean"]).max() < 1e-9


@pytest.mark.parametrize("name", ["scat_h2o_rhf_sto3g", "scat_oh_uhf_631g", "scat_h2_mom_631g"])
def test_input_file_scattering(name, tmp_path):
    """Job_Type = PROPERTY through the input-file runner: the GPU's own SCF states, then
    the table; state densities converged to 1e-8 move the intensities by less than 1e-6."""
    z = load(name)
    _, coords = molecule_for(z)
    lines = ['[%s]' % name, 'Method = "HF"', 'Basis_Sets = ["%s"]' % str(z["basis"]),
             'Multiplicity = %d' % int(z["multiplicity"]), 'Charge = 0', 'Coords_Units = "BOHR"',
             'Coords = %r' % coords, 'Reference = "%s"' % str(z["reference"]), 'Job_Type = "PROPERTY"',
             'Property_Type = "SCATTERING"', 'Property_Grid = %r' % [float(s) for s in z["grid"]]]
    if str(z["excitations"]):
        lines.append('Excitations = "%s"' % str(z["excitations"]))
    inp = tmp_path / "scat.inp"
    inp.write_text("\n".join(lines) + "\n")
    res = cli.run_file(str(inp), stream=open("/dev/null", "w"))[0]
    table = np.array(res["scattering"]["intensities"])
    assert np.abs(table - z["clean"]).max() < 1e-5
    text = (tmp_path / (name + ".out")).read_text()
    assert "Scattering patterns" in text
    torch.cuda.synchronize()
