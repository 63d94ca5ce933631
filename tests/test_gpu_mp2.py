"""MP2 AO->MO transform on BF16 tensor cores with FP64 accuracy (Ozaki splitting).

* the split GEMM against cuBLAS DGEMM on matrices whose rows span 8 decades;
* MP2 energies against the upstream fixtures (1e-8 Eh) and against the FP64-DGEMM
  transform on the full (H2O)16 / 6-31G workload (1e-8 Eh, a size-independent check).
"""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def test_ozaki_gemm_accuracy():
    from pychem_gb300.scf import ozaki_gemm
    g = torch.Generator(device="cuda").manual_seed(3)
    M, N, K, batch = 96, 200, 208, 3
    A = torch.randn(batch, M, K, dtype=torch.float64, device="cuda", generator=g)
    A *= torch.pow(10.0, -8 * torch.rand(batch, M, 1, dtype=torch.float64, device="cuda", generator=g))
    B = torch.randn(batch, K, N, dtype=torch.float64, device="cuda", generator=g)
    B *= torch.pow(10.0, -4 * torch.rand(batch, 1, N, dtype=torch.float64, device="cuda", generator=g))
    C = torch.empty(batch, M, N, dtype=torch.float64, device="cuda")
    ozaki_gemm(A, B, C, batch, M, N, K, (M * K, K, 1), (K * N, N, 1), M * N, nslice=6)
    ref = torch.bmm(A, B)
    scale = A.abs().amax(dim=2, keepdim=True) * B.abs().amax(dim=1, keepdim=True) * K
    rel = ((C - ref).abs() / scale).max().item()
    assert rel < 1e-12, rel
    # transposed operand layouts (unit stride along m for A, along k for B)
    At = A.transpose(1, 2).contiguous()   # [b][k][m]
    Bt = B.transpose(1, 2).contiguous()   # [b][n][k]
    C2 = torch.empty_like(C)
    ozaki_gemm(At, Bt, C2, batch, M, N, K, (M * K, 1, M), (K * N, 1, K), M * N, nslice=6)
    assert ((C2 - ref).abs() / scale).max().item() < 1e-12


@pytest.mark.parametrize("name", ["h2o_sto3g", "h2o_631g"])
def test_mp2_ozaki_fixture(golden_dir, name):
    from pychem_gb300.engine import GpuEngine
    from pychem_gb300.molecule import Molecule
    from pychem_gb300.scf import rhf, rmp2
    g = np.load(os.path.join(golden_dir, name + ".npz"))
    coords = [[str(s), float(z)] + list(map(float, xyz)) for s, z, xyz in zip(g["atoms"], g["charges"], g["coords_bohr"])]
    eng = GpuEngine(Molecule(coords, str(g["basis"]), units="BOHR")).prepare()
    r = rhf(eng)
    e_oz = rmp2(eng, r.C, r.eps, gemm="ozaki")
    e_64 = rmp2(eng, r.C, r.eps, gemm="fp64")
    assert abs(e_oz - e_64) < 1e-10
    assert abs(e_oz - float(g["E_mp2_corr"])) < 1e-8


def test_mp2_ozaki_water16():
    from pychem_gb300 import workloads as W
    from pychem_gb300.engine import GpuEngine
    from pychem_gb300.molecule import Molecule
    from pychem_gb300.scf import rhf, rmp2
    eng = GpuEngine(Molecule(W.water_cluster(), "6-31G")).prepare()
    r = rhf(eng)
    eri = eng.dense_eri()
    e_oz = rmp2(eng, r.C, r.eps, eri=eri, gemm="ozaki")
    e_64 = rmp2(eng, r.C, r.eps, eri=eri, gemm="fp64")
    assert abs(e_oz - e_64) < 1e-8, e_oz - e_64
