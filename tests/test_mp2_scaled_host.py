"""Spin-component-scaled MP2 (Methods/mp2.py:97-107) on CPU: pychem_gb300.scf.rmp2 /
ump2 with their FP64 transform path on CPU tensors, from the oracle's SCF orbitals,
against the reference's MP2, MP2-SCS and MP2-SOS correlation energies
(make_golden_mp2_scaled.py).  The pair-sum kernel (pcg_mp2_pair_sums) is replaced by
the same sums in torch, so that the host logic around it runs without a GPU."""
import json
import os

import numpy as np
import pytest
import torch

from oracle import oracle
from pychem_gb300.molecule import Molecule
from pychem_gb300.scf import MP2_SCALES, SCFResult, rmp2, ump2

HERE = os.path.dirname(os.path.abspath(__file__))
with open(os.path.join(HERE, "golden", "mp2_scaled.json")) as _fh:
    CASES = json.load(_fh)


def _torch_pair_sums(ovov, eo, ev):
    den = eo[:, None, None, None] - ev[None, :, None, None] + eo[None, None, :, None] - ev[None, None, None, :]
    t = ovov / den
    return float(torch.sum(ovov * t)), float(torch.sum(ovov.permute(0, 3, 2, 1) * t))


class _Eng:
    def __init__(self, mol):
        self.mol = mol


@pytest.mark.parametrize("name", sorted(CASES))
def test_scaled_mp2_matches_reference(name, monkeypatch):
    from pychem_gb300 import scf
    monkeypatch.setattr(scf, "mp2_pair_sums", _torch_pair_sums)
    case = CASES[name]
    mol = Molecule(case["coords"], case["basis"], multiplicity=case["multiplicity"])
    b = oracle.Basis([(a[0], a[1], *a[2]) for a in mol.atoms], mol.Basis)
    S, H = b.one_electron()
    eri = b.eri_dense()
    e_nuc = b.nuclear_repulsion()
    na, nb = mol.NAlphaElectrons, mol.NBetaElectrons
    eri_t = torch.tensor(eri)
    eng = _Eng(mol)
    if case["reference"] == "RHF":
        r = oracle.rhf(S, H, eri, na, e_nuc)
        assert abs(r["E"] - case["E_hf"]) < 1e-8
        run = lambda sc: rmp2(eng, torch.tensor(r["C"]), torch.tensor(r["eps"]), eri=eri_t, gemm="fp64", scale=sc)
    else:
        r = oracle.uhf(S, H, eri, na, nb, e_nuc)
        assert abs(r["E"] - case["E_hf"]) < 1e-8
        res = SCFResult(Ca=torch.tensor(r["Ca"]), Cb=torch.tensor(r["Cb"]), ea=torch.tensor(r["ea"]),
                        eb=torch.tensor(r["eb"]))
        run = lambda sc: ump2(eng, res, eri=eri_t, gemm="fp64", scale=sc)
    for method in ("MP2", "MP2-SCS", "MP2-SOS"):
        assert abs(run(MP2_SCALES[method]) - case[method]) < 1e-9, method
    # scale (1, 1) is plain MP2
    assert abs(run((1.0, 1.0)) - run(None)) < 1e-12
