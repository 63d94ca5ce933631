"""Jacobi eigensolver (FP64 batched, FP32 + FP64 refinement) against cuSOLVER."""
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def rand_sym(batch, n, seed, spread=1.0):
    g = torch.Generator(device="cuda").manual_seed(seed)
    M = torch.randn(batch, n, n, dtype=torch.float64, device="cuda", generator=g)
    A = (M + M.transpose(-1, -2)) * 0.5
    return A * spread


@pytest.mark.parametrize("n", [1, 2, 7, 13, 30, 57, 58, 64, 101, 136])
def test_fp64_jacobi_batched(n):
    from pychem_gb300 import eigen
    A = rand_sym(17, n, n)
    w, V = eigen.eigh(A)
    ref = torch.linalg.eigvalsh(A)
    assert (w - ref).abs().max().item() < 1e-12 * max(1.0, ref.abs().max().item())
    resid = A @ V - V * w.unsqueeze(-2)
    assert resid.abs().max().item() < 1e-12 * max(1.0, ref.abs().max().item())
    I = torch.eye(n, dtype=torch.float64, device="cuda")
    assert (V.transpose(-1, -2) @ V - I).abs().max().item() < 1e-13


def test_fp32_jacobi_accuracy():
    from pychem_gb300 import eigen
    A = rand_sym(3, 64, 5)
    w, V = eigen.jacobi(A, fp32=True)
    ref = torch.linalg.eigvalsh(A)
    assert (torch.sort(w, dim=-1)[0] - ref).abs().max().item() < 1e-3
    l, X = eigen.refine(A, V, steps=2)
    assert (torch.sort(l, dim=-1)[0] - ref).abs().max().item() < 1e-12


@pytest.mark.parametrize("n", [208, 298])
def test_refinement_from_previous_vectors(n):
    """SCF-iteration mode: after a small change of the matrix, refinement from the
    previous eigenvectors gives the projector onto a gapped lowest block to ~1e-11 and
    every eigenvalue outside a near-degenerate cluster to ~1e-10."""
    from pychem_gb300 import eigen
    g = torch.Generator(device="cuda").manual_seed(7)
    Q, _ = torch.linalg.qr(torch.randn(n, n, dtype=torch.float64, device="cuda", generator=g))
    lam = torch.linspace(-2.0, 5.0, n, dtype=torch.float64, device="cuda")
    lam[:16] = -20.5 + 1e-3 * torch.arange(16, dtype=torch.float64, device="cuda")   # core-like cluster
    nocc = 80
    lam[nocc:] += 0.5                                                                # HOMO-LUMO gap
    A = (Q * lam) @ Q.T
    w, V = eigen.eigh(A, exact=True)
    for scale in (1e-3, 1e-5):
        A2 = A + scale * rand_sym(1, n, 9)[0]
        w2, V2 = eigen.eigh(A2, X_prev=V, exact=False)
        ref2, U2 = torch.linalg.eigh(A2)
        P2 = V2[:, :nocc] @ V2[:, :nocc].T
        assert (P2 - U2[:, :nocc] @ U2[:, :nocc].T).abs().max().item() < 1e-11
        assert (w2[16:] - ref2[16:]).abs().max().item() < 1e-10
        # projector mode (what the SCF iterations use)
        w3, V3 = eigen.eigh(A2, X_prev=V, exact=False, nocc=nocc)
        P3 = V3[:, :nocc] @ V3[:, :nocc].T
        assert (P3 - U2[:, :nocc] @ U2[:, :nocc].T).abs().max().item() < 1e-11
        I = torch.eye(n, dtype=torch.float64, device="cuda")
        assert (V2.T @ V2 - I).abs().max().item() < 1e-12


@pytest.mark.parametrize("n", [13, 82, 181, 182, 190])
def test_fp32_eigh_with_previous_vectors(n):
    """FP32 Jacobi (V in shared memory up to n = 182, in global memory above): from
    scratch and from nearby previous eigenvectors, eigenvalues to FP32 accuracy and an
    orthogonal eigenvector matrix."""
    from pychem_gb300 import eigen
    A = rand_sym(4, n, 11)
    ref = torch.linalg.eigvalsh(A)
    scale = max(1.0, ref.abs().max().item())
    w, V = eigen.eigh32(A)
    assert V.dtype == torch.float32
    assert (w - ref).abs().max().item() < 2e-5 * scale * n ** 0.5
    I = torch.eye(n, dtype=torch.float32, device="cuda")
    assert (V.transpose(-1, -2) @ V - I).abs().max().item() < 2e-5 * n ** 0.5
    A2 = A + 1e-3 * rand_sym(4, n, 12)
    ref2 = torch.linalg.eigvalsh(A2)
    w2, V2 = eigen.eigh32(A2, X_prev=V)
    assert (w2 - ref2).abs().max().item() < 2e-5 * scale * n ** 0.5
    resid = A2.float() @ V2 - V2 * w2.float().unsqueeze(-2)
    assert resid.abs().max().item() < 1e-4 * scale * n ** 0.5


@pytest.mark.parametrize("M,N,K", [(1, 1, 1), (7, 13, 5), (208, 208, 208), (208, 80, 208), (33, 65, 97),
                                   (298, 298, 298), (64, 1, 300)])
@pytest.mark.parametrize("ta,tb", [(False, False), (True, False), (False, True), (True, True)])
def test_dgemm_against_torch(M, N, K, ta, tb):
    """pcg_dgemm (double-buffered 8 x 8 tiles, K steps of 32) against torch's FP64 matmul,
    with transposes through strides, alpha/beta, and a batch of 3."""
    from pychem_gb300 import dense
    g = torch.Generator(device="cuda").manual_seed(M * 7 + N * 3 + K)
    A = torch.randn(3, K, M, dtype=torch.float64, device="cuda", generator=g)
    B = torch.randn(3, N, K, dtype=torch.float64, device="cuda", generator=g)
    A = A.transpose(-1, -2) if not ta else A           # op(A) is M x K either way
    A = A if not ta else A.contiguous()
    B = B.transpose(-1, -2) if not tb else B
    opA = A.transpose(-1, -2) if ta else A
    opB = B.transpose(-1, -2) if tb else B
    C0 = torch.randn(3, M, N, dtype=torch.float64, device="cuda", generator=g)
    out = C0.clone()
    dense.mm(A, B, ta=ta, tb=tb, out=out, alpha=0.5, beta=-2.0)
    ref = 0.5 * (opA @ opB) - 2.0 * C0
    assert (out - ref).abs().max().item() < 1e-12 * max(1.0, K ** 0.5)
