"""GPU energies at the two large benchmark configurations against the CPU oracle
(tests/golden/configs.json, made by tests/golden/make_golden_configs.py with the
oracle's packed store, whose restatement tests/test_oracle_packed.py and
tests/test_oracle_golden.py pin to the reference):

* (H2O)16 / 6-31G, 208 AO (the headline workload): RHF total energy and RMP2
  correlation energy through the tensor-core (Ozaki) transforms, each within 1e-8 Eh;
* C12H26 / cc-pVDZ, 298 AO: RHF total energy in plain FP64 and in mixed precision
  (quartets with Schwarz bound below 1e-4 in FP32), each within 1e-8 Eh.
"""
import json
import os

import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = 1e-8   # Eh


def _fixture(golden_dir, key):
    from pychem_gb300.molecule import Molecule
    d = json.load(open(os.path.join(golden_dir, "configs.json")))[key]
    return d, Molecule(d["atoms_bohr"], d["basis"], units="BOHR")


def test_water16_rhf_mp2_against_oracle(golden_dir):
    from pychem_gb300.engine import GpuEngine
    from pychem_gb300.scf import rhf, rmp2
    d, mol = _fixture(golden_dir, "c2_water16_631g")
    eng = GpuEngine(mol).prepare()
    assert eng.nbf == d["nbf"]
    r = rhf(eng)
    assert r.converged
    assert abs(r.E - d["E_rhf"]) < TOL, (r.E, d["E_rhf"])
    e2 = rmp2(eng, r.C, r.eps)
    assert abs(e2 - d["E_mp2_corr"]) < TOL, (e2, d["E_mp2_corr"])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_c12h26_rhf_against_oracle(golden_dir, precision):
    from pychem_gb300.engine import GpuEngine
    from pychem_gb300.scf import rhf
    d, mol = _fixture(golden_dir, "c3_c12h26_ccpvdz")
    eng = GpuEngine(mol, precision=precision, fp32_below=1e-4).prepare()
    assert eng.nbf == d["nbf"]
    r = rhf(eng)
    assert r.converged
    assert abs(r.E - d["E_rhf"]) < TOL, (precision, r.E, d["E_rhf"], r.E - d["E_rhf"])
