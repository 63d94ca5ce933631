"""MP2 AO->MO transform on the tcgen05 tensor cores with FP64 accuracy (Ozaki digit
slices, every level in one kernel; the kernel itself is tested in test_gpu_oz_tc.py):

* MP2 energies against the upstream fixtures (1e-8 Eh) and against the FP64-DGEMM
  transform (1e-10 Eh), also on the full (H2O)16 / 6-31G workload.
"""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["h2o_sto3g", "h2o_631g"])
def test_mp2_tc_fixture(golden_dir, name):
    from pychem_gb300.engine import GpuEngine
    from pychem_gb300.molecule import Molecule
    from pychem_gb300.scf import rhf, rmp2
    g = np.load(os.path.join(golden_dir, name + ".npz"))
    coords = [[str(s), float(z)] + list(map(float, xyz)) for s, z, xyz in zip(g["atoms"], g["charges"], g["coords_bohr"])]
    eng = GpuEngine(Molecule(coords, str(g["basis"]), units="BOHR")).prepare()
    r = rhf(eng)
    e_oz = rmp2(eng, r.C, r.eps, gemm="tc")
    e_64 = rmp2(eng, r.C, r.eps, gemm="fp64")
    assert abs(e_oz - e_64) < 1e-10
    assert abs(e_oz - float(g["E_mp2_corr"])) < 1e-8


def test_mp2_tc_water16():
    from pychem_gb300 import workloads as W
    from pychem_gb300.engine import GpuEngine
    from pychem_gb300.molecule import Molecule
    from pychem_gb300.scf import rhf, rmp2
    eng = GpuEngine(Molecule(W.water_cluster(), "6-31G")).prepare()
    r = rhf(eng)
    eri = eng.dense_eri()
    e_oz = rmp2(eng, r.C, r.eps, eri=eri, gemm="tc")
    e_64 = rmp2(eng, r.C, r.eps, eri=eri, gemm="fp64")
    assert abs(e_oz - e_64) < 1e-10, e_oz - e_64


def test_compact_pair_tensor_water16():
    """The compact pair-packed tensor holds exactly the rows of the full pair-packed one
    for the AO pairs in some off-diagonal stored quartet; the rows it leaves out are
    below 1e-14; MP2 from it matches the FP64 transform of the full tensor."""
    from pychem_gb300 import workloads as W
    from pychem_gb300.engine import GpuEngine
    from pychem_gb300.molecule import Molecule
    from pychem_gb300.scf import rhf, rmp2
    eng = GpuEngine(Molecule(W.water_cluster(), "6-31G")).prepare()
    n = eng.nbf
    full = eng.dense_eri_pairs()
    Ec, pmap, rows = eng.dense_eri_pairs(compact=True)
    pm = pmap.to(torch.int64)
    keep = pm >= 0
    assert rows == int(keep.sum()) and 0 < rows < n * (n + 1) // 2
    assert torch.equal(pm[keep], torch.arange(rows, device=pm.device))
    assert torch.equal(Ec, full[keep])
    assert float(full[~keep].abs().max()) < 1e-14
    del full
    r = rhf(eng)
    e_c = rmp2(eng, r.C, r.eps, eri=(Ec, pmap, rows), gemm="tc")
    del Ec
    e_64 = rmp2(eng, r.C, r.eps, gemm="fp64")
    assert abs(e_c - e_64) < 1e-10, e_c - e_64
