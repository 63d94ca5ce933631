"""Batched RHF of a molecule ensemble against the one-molecule path.

Seeded perturbed H2O, NH3, CH4, HF, CH3OH, C2H6 in 6-31G (11-30 AO, uneven sizes):
per-molecule S and H blocks within 1e-10 and RHF energies within 1e-8 Eh of the
single-molecule engine (itself pinned to the upstream reference), plus one molecule
against the CPU oracle directly.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ensemble():
    from pychem_gb300 import workloads as W
    from pychem_gb300.ensemble import EnsembleEngine, rhf_batched
    from pychem_gb300.molecule import Molecule
    mols = [Molecule(c, "6-31G") for c in W.ensemble(n=12, seed=11)]
    eng = EnsembleEngine(mols).prepare()
    res = rhf_batched(eng)
    return mols, eng, res


def test_one_electron_blocks(ensemble):
    from pychem_gb300.engine import GpuEngine
    mols, eng, res = ensemble
    for m in (0, 4, 5, 11):
        single = GpuEngine(mols[m])
        S, H = single.one_electron()
        n = mols[m].NOrbitals
        assert (eng.S[m, :n, :n] - S).abs().max().item() < 1e-10
        assert (eng.H[m, :n, :n] - H).abs().max().item() < 1e-10


def test_energies_match_single_molecule_path(ensemble):
    from pychem_gb300.engine import GpuEngine
    from pychem_gb300.scf import rhf
    mols, eng, res = ensemble
    assert res.converged.all()
    for m, mol in enumerate(mols):
        r = rhf(GpuEngine(mol).prepare())
        assert abs(res.E[m] - r.E) < 1e-8, (m, res.E[m] - r.E)


def test_one_member_against_oracle(ensemble):
    from oracle import oracle as O
    mols, eng, res = ensemble
    m = 3   # HF molecule
    mol = mols[m]
    b = O.Basis([(a[0], a[1], *a[2]) for a in mol.atoms], "6-31G")
    S, H = b.one_electron()
    ref = O.rhf(S, H, b.eri_dense(), mol.NAlphaElectrons, b.nuclear_repulsion())
    assert abs(res.E[m] - ref["E"]) < 1e-8


def test_compaction_changes_nothing(ensemble):
    """Cutting the quartet lists down to the active molecules (here after every
    convergence) gives the same energies and iteration counts as never cutting them,
    and the engine's full lists come back afterwards."""
    from pychem_gb300.ensemble import rhf_batched
    mols, eng, res = ensemble
    n_before = sum(n for rec in eng.classes.values() for (_, n) in rec.values())
    r_never = rhf_batched(eng, compact=0.0)
    r_always = rhf_batched(eng, compact=1.0)
    assert sum(n for rec in eng.classes.values() for (_, n) in rec.values()) == n_before
    assert (r_never.iterations == r_always.iterations).all()
    assert np.abs(r_never.E - r_always.E).max() < 1e-12
    assert np.abs(r_never.E - res.E).max() < 1e-12
    assert (r_always.D - r_never.D).abs().max().item() < 1e-10


def test_fp32_dense_phase_reaches_the_fp64_state(ensemble):
    """Mixed-precision dense steps (FP32 until the DIIS residual RMS drops below 1e-4)
    converge every molecule to the FP64 energies."""
    from pychem_gb300.ensemble import rhf_batched
    mols, eng, res = ensemble
    trace = []
    r = rhf_batched(eng, dense_fp32_until=1e-4, trace=trace)
    assert r.converged.all()
    assert np.abs(r.E - res.E).max() < 1e-9
    assert trace[0][2] == len(mols)          # every molecule starts in FP32
    assert trace[-1][2] == 0
