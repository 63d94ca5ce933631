"""Learned initial guess: forward/backward kernels against the FP64 CPU oracle, and the
trained network's effect on the SCF (the SAD-guess SCF stays the reference result)."""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def test_forward_backward_against_oracle():
    from oracle import mlp_oracle as O
    from pychem_gb300.learned.mlp import PairMLP
    net = PairMLP(seed=3)
    g = torch.Generator(device="cuda").manual_seed(1)
    M = 300
    X = torch.randn(M, net.dims[0], device="cuda", generator=g)
    T = torch.randn(M, net.dims[-1], device="cuda", generator=g)
    mask = (torch.rand(M, net.dims[-1], device="cuda", generator=g) > 0.3).float()
    Y, cache = net.forward(X, keep=True)
    loss, dY = net.loss_grad(Y, T, mask)
    grads = net.backward(dY, cache)
    Ws = [w.to(torch.float64).cpu().numpy() for w in net.Wb]       # the BF16 weights the kernels use
    bs = [b.double().cpu().numpy() for b in net.b]
    l_ref, Y_ref, g_ref = O.loss_and_grads(X.double().cpu().numpy(), T.double().cpu().numpy(),
                                           mask.double().cpu().numpy(), Ws, bs)
    assert np.abs(Y.cpu().numpy() - Y_ref).max() < 1e-4 * max(1.0, np.abs(Y_ref).max())
    assert abs(float(loss) - l_ref) < 1e-4 * l_ref
    for (dW, db), (rW, rb) in zip(grads, g_ref):
        assert np.abs(dW.cpu().numpy() - rW).max() < 2e-4 * max(1e-3, np.abs(rW).max())
        assert np.abs(db.cpu().numpy() - rb).max() < 2e-4 * max(1e-3, np.abs(rb).max())


def test_training_reduces_loss():
    """Dataset from converged batched SCFs of 96 generated molecules, a few epochs:
    both the off-diagonal slot loss and the diagonal-correction loss fall."""
    from pychem_gb300.learned.molgen import molecules
    from pychem_gb300.learned.train import build_dataset, chunks_by_size, train
    from pychem_gb300.molecule import Molecule
    mols = [Molecule(c, "6-31G") for c in molecules(96, seed=5)]
    pairs, atoms, n = build_dataset(mols, chunks_by_size(mols))
    assert n == 96
    net, hist = train(pairs, atoms, n, epochs=8, mols_per_batch=12, lr=2e-3)
    assert hist[-1][0] < 0.5 * hist[0][0]
    assert hist[-1][1] < 0.5 * hist[0][1]


WEIGHTS = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "pychem_gb300", "data",
                       "learned_guess_631g.npz")


@pytest.mark.skipif(not os.path.exists(WEIGHTS), reason="no trained weights committed")
def test_learned_guess_gain_and_energy():
    """On held-out molecules (seed 2, not seen in training) the learned guess reaches
    the SAD-guess energies to 1e-8 Eh in fewer SCF iterations on average."""
    from pychem_gb300.ensemble import EnsembleEngine, rhf_batched
    from pychem_gb300.learned.mlp import PairMLP
    from pychem_gb300.learned.molgen import molecules
    from pychem_gb300.learned.train import guess_density
    from pychem_gb300.molecule import Molecule
    net = PairMLP.load(WEIGHTS)
    mols = [Molecule(c, "6-31G") for c in molecules(128, seed=2)]
    eng = EnsembleEngine(mols).prepare()
    r_sad = rhf_batched(eng, guess="sad")
    r_nn = rhf_batched(eng, D0=guess_density(net, mols, eng))
    assert r_sad.converged.all() and r_nn.converged.all()
    assert np.abs(r_nn.E - r_sad.E).max() < 1e-8
    assert r_nn.iterations.mean() < r_sad.iterations.mean()
