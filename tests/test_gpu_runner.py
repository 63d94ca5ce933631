"""The input-file runner's multi-basis bootstrap, MO text files and SCS/SOS-MP2 on the
GPU: the same cases and bars as the CPU tests (tests/test_bootstrap_host.py,
tests/test_mp2_scaled_host.py), with the GPU engine, SCFs and tensor-core MP2
transforms instead of the oracle standing in for them.

* cli.run_bootstrap over several basis sets (orbitals fitted with upstream's
  bookkeeping seed the later bases' MOM states): per-basis state energies against the
  reference's own multi-basis runs (ground states 1e-8 Eh, MOM states 1e-5 where the
  reference converged them, else 1e-3);
* Dump_MOs files and the READ guess that restarts from them;
* MP2, MP2-SCS and MP2-SOS correlation energies (RHF and UHF) against the reference's
  (make_golden_mp2_scaled.py), 1e-8 Eh.
"""
import json
import os
import sys

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import test_bootstrap_host as host  # noqa: E402  (cases, options and the reference residual)


@pytest.mark.parametrize("name", [n for n in sorted(host.BOOT) if n.startswith("boot_")])
def test_bootstrap_energies_on_gpu(name, tmp_path):
    from pychem_gb300 import cli
    case = host.BOOT[name]
    res = cli.run_bootstrap(name, host._opts(case), lambda line: None, str(tmp_path))
    got = [(pb["basis"], k, e) for pb in res["per_basis"] for k, e in enumerate(pb["E_hf"])]
    assert len(got) == len(case["calls"])
    for call, ((basis, k, e), (rb, rk, re_)) in enumerate(zip(got, case["calls"])):
        assert basis.replace("-", "").upper() == rb and k == rk
        if k == 0:
            assert abs(e - re_) < 1e-8, (basis, k, e, re_)
        else:
            converged = host.reference_residual(name, call, basis, case["coords"]) < 1e-5
            assert abs(e - re_) < (1e-5 if converged else 1e-3), (basis, k, e, re_)


def test_dump_and_read_mos_on_gpu(tmp_path):
    from pychem_gb300 import cli
    case = host.BOOT["boot_h2_mom_sto3g_631g"]
    opts = dict(host._opts(case), DUMP_MOS=True)
    res = cli.run_bootstrap("dump", opts, lambda line: None, str(tmp_path))
    for basis in ("STO3G", "631G"):
        for k in (0, 1):
            for spin in ("alpha", "beta"):
                assert (tmp_path / ("%s_%d.%s_MOs" % (basis, k, spin))).exists()
    opts = dict(host._opts(case), BASIS_SETS=["6-31G"], SCF_GUESS="READ", MO_READ_BASIS="6-31G", MO_READ_STATE=[0, 1])
    again = cli.run_bootstrap("read", opts, lambda line: None, str(tmp_path))
    e_dump = res["per_basis"][1]["E_hf"]
    e_read = again["per_basis"][0]["E_hf"]
    assert abs(e_read[0] - e_dump[0]) < 1e-8 and abs(e_read[1] - e_dump[1]) < 1e-6
    assert again["per_basis"][0]["iterations"][0] <= 3


with open(os.path.join(HERE, "golden", "mp2_scaled.json")) as _fh:
    MP2_CASES = json.load(_fh)


@pytest.mark.parametrize("name", sorted(MP2_CASES))
def test_scaled_mp2_on_gpu(name):
    from pychem_gb300.engine import GpuEngine
    from pychem_gb300.molecule import Molecule
    from pychem_gb300.scf import MP2_SCALES, rhf, rmp2, uhf, ump2
    case = MP2_CASES[name]
    mol = Molecule(case["coords"], case["basis"], multiplicity=case["multiplicity"])
    eng = GpuEngine(mol).prepare()
    if case["reference"] == "RHF":
        r = rhf(eng)
        run = lambda sc: rmp2(eng, r.C, r.eps, scale=sc)
    else:
        r = uhf(eng)
        run = lambda sc: ump2(eng, r, scale=sc)
    assert r.converged and abs(r.E - case["E_hf"]) < 1e-8
    for method in ("MP2", "MP2-SCS", "MP2-SOS"):
        assert abs(run(MP2_SCALES[method]) - case[method]) < 1e-8, method
