"""Symmetric eigensolver for the SCF on the GPU (replaces numpy.linalg.eigh of
``Methods/hartree_fock.py:172-175,226``).

* n <= 136: parallel cyclic Jacobi in FP64, one CTA per matrix (pcg_jacobi_eigh),
  batched over any leading dimension.
* larger n, inside SCF iterations: FP64 iterative refinement of the previous
  iteration's eigenvectors (T. Ogita and K. Aishima, "Iterative refinement for
  symmetric eigenvalue decomposition", Japan J. Indust. Appl. Math. 35 (2018)
  1007-1035, Algorithm 1): four FP64 GEMMs per step instead of a tridiagonalisation.
* the FP32 variant of the Jacobi kernel (``jacobi(..., fp32=True)``) gives FP32-accurate
  starting vectors for the same refinement.
Eigenvalues are returned ascending with matching eigenvector columns.
"""
import ctypes

import torch

from . import _lib

FP64_JACOBI_MAX_N = 136

# counts of eigh calls by route (exact library solve, refinement, refinement rejected)
stats = {"exact": 0, "refined": 0, "fallback": 0}


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def jacobi(A, fp32=False, max_sweeps=40, tol=None):
    """Unsorted eigenpairs of a batch of symmetric matrices (..., n, n), FP64 input and
    FP64 output (the FP32 variant's vectors converted)."""
    w, V = _jacobi(A, fp32, max_sweeps, tol)
    return w, V.to(torch.float64)


def eigh32(A, X_prev=None):
    """Ascending FP32-accurate eigenpairs of symmetric A (..., n, n), n <= 334, with the
    FP32 Jacobi kernel; with X_prev (orthogonal, float32) the kernel works on
    X_prev^T A X_prev, which is nearly diagonal between SCF iterations.  Returns
    (w float64, V float32)."""
    A = A.to(torch.float32)
    if X_prev is not None:
        Ap = X_prev.transpose(-1, -2) @ A @ X_prev
        w, V = _jacobi(Ap.to(torch.float64), True, 40, None)
        return _sort(w, X_prev @ V)
    return _sort(*_jacobi(A.to(torch.float64), True, 40, None))


def _jacobi(A, fp32, max_sweeps, tol):
    shape = A.shape
    n = shape[-1]
    A2 = A.reshape(-1, n, n).contiguous()
    batch = A2.shape[0]
    m = n + (n & 1)
    dt = torch.float32 if fp32 else torch.float64
    w = torch.empty(batch, n, dtype=torch.float64, device=A.device)
    V = torch.empty(batch, m, m, dtype=dt, device=A.device)
    if tol is None:
        tol = 2e-7 if fp32 else 1e-15
    _lib.call("pcg_jacobi_eigh", batch, n, ctypes.c_void_p(A2.data_ptr()), ctypes.c_void_p(w.data_ptr()),
              ctypes.c_void_p(V.data_ptr()), 1 if fp32 else 0, None, max_sweeps, float(tol), None, _stream())
    return w.reshape(shape[:-1]), V[:, :n, :n].reshape(shape)


def _sort(w, V):
    w, idx = torch.sort(w, dim=-1)
    V = torch.gather(V, -1, idx.unsqueeze(-2).expand_as(V))
    return w, V


def refine(A, X, steps=2):
    """Ogita-Aishima refinement of approximate eigenvectors X of symmetric A (FP64).
    Pairs with |l_i - l_j| <= delta, delta = 2 (||S - diag(l)||_F + ||A||_F ||R||_F) (the
    paper's 2-norms bounded by Frobenius norms), are only re-orthogonalised: from an
    FP32 start, vectors inside a cluster of near-degenerate eigenvalues stay mixed
    within the cluster while everything separated by more than delta converges
    quadratically.  The SCF needs only the occupied-space projector, which a mixed
    occupied (or virtual) cluster leaves unchanged."""
    n = A.shape[-1]
    I = torch.eye(n, dtype=torch.float64, device=A.device)
    lam = None
    for _ in range(steps):
        R = I - X.transpose(-1, -2) @ X
        S = X.transpose(-1, -2) @ (A @ X)
        lam = torch.diagonal(S, dim1=-2, dim2=-1) / (1.0 - torch.diagonal(R, dim1=-2, dim2=-1))
        off = S - torch.diag_embed(lam)
        nA = A.flatten(-2).norm(dim=-1)
        delta = 2.0 * (off.flatten(-2).norm(dim=-1) + nA * R.flatten(-2).norm(dim=-1))
        dl = lam.unsqueeze(-2) - lam.unsqueeze(-1)          # [i, j] = lam_j - lam_i
        sep = dl.abs() > delta.unsqueeze(-1).unsqueeze(-1)
        E = torch.where(sep, (S + lam.unsqueeze(-2) * R) / torch.where(sep, dl, torch.ones_like(dl)), 0.5 * R)
        X = X + X @ E
    return lam, X


def refine_projector(A, X, nocc, steps=2):
    """Refinement that only decouples the first nocc columns (occupied) from the rest
    (virtual): Ogita-Aishima corrections for occupied-virtual pairs, separated by at
    least the HOMO-LUMO gap, and re-orthonormalisation (E = R/2) inside each block.
    Converges quadratically in the occupied-space projector regardless of
    near-degeneracies inside the blocks."""
    n = A.shape[-1]
    I = torch.eye(n, dtype=torch.float64, device=A.device)
    occ = torch.zeros(n, dtype=torch.bool, device=A.device)
    occ[:nocc] = True
    ov = occ.unsqueeze(-1) ^ occ.unsqueeze(-2)
    lam = None
    for _ in range(steps):
        R = I - X.transpose(-1, -2) @ X
        S = X.transpose(-1, -2) @ (A @ X)
        lam = torch.diagonal(S) / (1.0 - torch.diagonal(R))
        dl = lam.unsqueeze(-2) - lam.unsqueeze(-1)
        E = torch.where(ov, (S + lam.unsqueeze(-2) * R) / torch.where(ov, dl, torch.ones_like(dl)), 0.5 * R)
        X = X + X @ E
    return lam, X


def eigh(A, X_prev=None, refine_steps=2, exact=True, check_tol=1e-10, nocc=None):
    """Ascending eigenvalues and eigenvectors of symmetric FP64 A (..., n, n).

    n <= 136: batched FP64 Jacobi (exact to rounding; the small-molecule ensemble).
    Larger n, exact=False and a previous eigenvector matrix X_prev (consecutive SCF
    iterations): FP64 refinement starting from X_prev -- quadratic convergence for
    every pair separated by more than the refinement threshold; pairs inside a
    near-degenerate cluster may stay rotated within it, which leaves the occupied-
    space projector unchanged.  The result is checked (orthogonality and the
    residual of separated pairs); on failure, and whenever exact=True or there is no
    X_prev, the library solver (cuSOLVER) is used."""
    n = A.shape[-1]
    if n <= FP64_JACOBI_MAX_N:
        if X_prev is not None:
            Ap = X_prev.transpose(-1, -2) @ A @ X_prev
            w, V = jacobi(Ap)
            return _sort(w, X_prev @ V)
        return _sort(*jacobi(A))
    if exact or X_prev is None:
        stats["exact"] += 1
        return torch.linalg.eigh(A)
    I = torch.eye(n, dtype=torch.float64, device=A.device)
    if nocc is not None:
        # SCF iterations: only the occupied-space projector matters.  Refine in rounds
        # of refine_steps steps until the vectors are orthonormal, the occupied block is
        # decoupled (max |(X^T A X)_ov| <= check_tol |A|) and gapped; after three rounds
        # fall back to the exact solver.
        X = X_prev
        scale = float(A.abs().amax())
        ok = False
        for _ in range(3):
            w, X = refine_projector(A, X, nocc, steps=refine_steps)
            orth = (X.transpose(-1, -2) @ X - I).abs().amax()
            ov = (X[:, :nocc].transpose(-1, -2) @ (A @ X[:, nocc:])).abs().amax()
            gap = w[nocc:].min() - w[:nocc].max()
            chk = torch.stack([orth, ov, -gap]).cpu()
            if float(chk[0]) <= check_tol and float(chk[1]) <= check_tol * max(scale, 1.0) and float(chk[2]) < 0.0:
                ok = True
                break
        if not ok:
            stats["fallback"] += 1
            return torch.linalg.eigh(A)
        stats["refined"] += 1
        wo, io = torch.sort(w[:nocc])
        wv, iv = torch.sort(w[nocc:])
        return torch.cat([wo, wv]), torch.cat([X[:, :nocc][:, io], X[:, nocc:][:, iv]], dim=1)
    w, X = refine(A, X_prev, steps=refine_steps)
    orth = (X.transpose(-1, -2) @ X - I).abs().amax()
    if float(orth) > check_tol:
        return torch.linalg.eigh(A)
    return _sort(w, X)
