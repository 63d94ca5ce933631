"""Symmetric eigensolver for the SCF on the GPU (replaces numpy.linalg.eigh of
``Methods/hartree_fock.py:172-175,226``), on the library's own kernels only:

* n <= 136: parallel cyclic Jacobi in FP64, one CTA per matrix (pcg_jacobi_eigh),
  batched over any leading dimension.
* larger n: the FP32 variant of the Jacobi kernel (FP32-accurate vectors, n <= 334),
  then FP64 iterative refinement (T. Ogita and K. Aishima, "Iterative refinement for
  symmetric eigenvalue decomposition", Japan J. Indust. Appl. Math. 35 (2018)
  1007-1035, Algorithm 1) with the library's FP64 GEMM (pcg_dgemm) and correction
  kernel (pcg_oa_correction).  Inside SCF iterations the refinement starts from the
  previous iteration's vectors and only decouples the occupied columns; exact
  solutions slice the spectrum at gaps into parts of at most 136, which the FP64
  Jacobi kernel finishes, so near-degenerate clusters are resolved exactly.
Eigenvalues are returned ascending with matching eigenvector columns.
"""
import ctypes

import torch

from . import _lib, dense

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


def eigh32_own(A, X_prev=None, tol=1e-5, max_sweeps=12):
    """eigh32 for one matrix (n, n) with FP64 in and out and the library GEMM for the
    rotations into and out of X_prev's basis: FP32-accurate eigenpairs, ascending.
    The Jacobi sweeps stop at an off-diagonal norm of tol (relative): the result
    only seeds FP64 refinement, which needs vectors good to well inside the gaps it
    separates, not FP32's last digit."""
    A = A.to(torch.float64)
    if X_prev is not None:
        Xp = X_prev.to(torch.float64)
        Ap = dense.mm(Xp, dense.mm(A, Xp), ta=True)
        w, V = _jacobi(Ap, True, max_sweeps, tol)
        return _sort(w, dense.mm(Xp, V.to(torch.float64)))
    w, V = _jacobi(A, True, max_sweeps, tol)
    return _sort(w, V.to(torch.float64))


def orthonormalize(X, steps=2):
    """X <- X + X (I - X^T X) / 2, twice: columns orthonormal to FP64 rounding from
    FP32-orthonormal ones (Newton-Schulz for the polar factor)."""
    for _ in range(steps):
        R, _ = _rs(None, X, need_s=False)
        X = _step(X, 0.5 * R)
    return X


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


def _rs(A, X, need_s=True):
    """R = I - X^T X and S = X^T A X on the library GEMM."""
    n = X.shape[-1]
    R = torch.eye(n, dtype=torch.float64, device=X.device)
    dense.mm(X, X, ta=True, out=R, alpha=-1.0, beta=1.0)
    S = dense.mm(X, dense.mm(A, X), ta=True) if need_s else None
    return R, S


def _step(X, E):
    Xn = X.clone()
    return dense.mm(X, E, out=Xn, beta=1.0)


def refine(A, X, steps=2):
    """Ogita-Aishima refinement of approximate eigenvectors X of symmetric A (FP64).
    Pairs with |l_i - l_j| <= delta, delta = 2 (||S - diag(l)||_F + ||A||_F ||R||_F) (the
    paper's 2-norms bounded by Frobenius norms), are only re-orthogonalised: vectors
    inside a cluster of near-degenerate eigenvalues stay mixed within the cluster
    while everything separated by more than delta converges quadratically.  Batched
    over a leading dimension; no host round trip."""
    if X.dim() == 3:
        out = [refine(A[k] if A.dim() == 3 else A, X[k], steps) for k in range(X.shape[0])]
        return torch.stack([o[0] for o in out]), torch.stack([o[1] for o in out])
    X = X.to(torch.float64)
    lam = torch.empty(X.shape[-1], dtype=torch.float64, device=X.device)
    nA = torch.linalg.vector_norm(A)
    for _ in range(steps):
        R, S = _rs(A, X)
        l = torch.diagonal(S) / (1.0 - torch.diagonal(R))
        delta = 2.0 * (torch.linalg.vector_norm(S - torch.diag(l)) + nA * torch.linalg.vector_norm(R))
        E = dense.oa_correction(S, R, 0, 1, delta=delta, lam=lam)
        X = _step(X, E)
    return lam.clone(), X


def refine_projector(A, X, nocc, steps=2, check=False, ortho_steps=1):
    """Refinement that only decouples the first nocc columns (occupied) from the rest
    (virtual): Ogita-Aishima corrections for occupied-virtual pairs, separated by at
    least the HOMO-LUMO gap, and re-orthonormalisation (E = R/2) inside each block, so
    the columns stay orthonormal to rounding.  Quadratic in the occupied-space
    projector while the blocks of X^T A X are nearly diagonal (X close to
    eigenvectors); as they drift from diagonal between SCF iterations it becomes a
    fast linear iteration.  With check=True also returns a device
    vector (orthogonality error, largest occupied-virtual coupling, minus the gap
    between the blocks' Rayleigh quotients) of the refined vectors."""
    lam = torch.empty(X.shape[-1], dtype=torch.float64, device=X.device)
    for _ in range(steps):
        R, S = _rs(A, X)
        E = dense.oa_correction(S, R, nocc, 0, lam=lam)
        X = _step(X, E)
    # the occupied-virtual rotations of large steps leave O(E^2) non-orthogonality;
    # a Newton-Schulz step X <- X + X (I - X^T X)/2 removes it quadratically
    X = orthonormalize(X, steps=ortho_steps)
    if not check:
        return lam, X
    R, S = _rs(A, X)
    d = torch.diagonal(S)
    chk = torch.stack([R.abs().amax(), S[:nocc, nocc:].abs().amax(), d[:nocc].amax() - d[nocc:].amin()])
    return lam, X, chk


EXACT_BLOCK = 64    # exact_eigh finishes blocks up to this size with the FP64 Jacobi kernel


def _split_point(w, n, base=EXACT_BLOCK):
    """Where to slice an ascending spectrum of size n > base: the largest gap among the
    positions that leave both parts at most base long, or, when that window is
    narrower than a quarter of n, among the middle half."""
    lo, hi = max(1, n - base), min(n - 1, base)
    if hi - lo < n // 4:
        lo, hi = n // 4, (3 * n) // 4
    gaps = w[lo:hi + 1] - w[lo - 1:hi]
    return lo + int(torch.argmax(gaps))


def exact_eigh(A, X_prev=None, steps=4):
    """Eigenpairs of one symmetric A to FP64 accuracy on the library's kernels, by
    spectrum slicing (exact_eigh_many with one matrix)."""
    return exact_eigh_many([A], [X_prev], steps=steps)[0]


def _padded(mats, m):
    """(len(mats), m, m) with each matrix in the top-left corner and, below it, a
    diagonal of one value above every spectrum: the padding rows are exact, decoupled
    eigenvectors that sort last and that the Jacobi kernel never rotates."""
    # one above the largest Gershgorin upper bound (not far above it: the padding adds
    # to the norm that the Jacobi kernel's stopping test is relative to)
    big = max(float((torch.diagonal(a) + a.abs().sum(dim=1) - torch.diagonal(a).abs()).amax()) for a in mats) + 1.0
    out = torch.zeros(len(mats), m, m, dtype=torch.float64, device=mats[0].device)
    for k, a in enumerate(mats):
        n = a.shape[0]
        out[k, :n, :n] = a
        if n < m:
            out[k, n:, n:].diagonal().fill_(big)
    return out


def exact_eigh_many(As, X_prevs=None, steps=4):
    """Eigenpairs of several symmetric matrices to FP64 accuracy, by spectrum slicing,
    with every Jacobi stage one batched launch (one CTA or a few per matrix, all
    matrices side by side on the GPU):

    * FP32 Jacobi vectors for every matrix (from X_prev when given);
    * a matrix above 64 is split at the largest gap that keeps both parts at most 64
      (or in the middle half), projector refinement decouples the two invariant
      subspaces in FP64, and each part's projected matrix -- nearly diagonal already,
      in the FP32 vectors' basis, its diagonal ordering the part's spectrum -- is
      split the same way while above 64;
    * every part of at most 64 is finished by the FP64 Jacobi kernel, which needs
      few sweeps from nearly diagonal, all parts in one batched launch.

    Near-degenerate clusters end up inside one part, where Jacobi resolves them.
    Returns [(w ascending, V)] in the order of As."""
    if X_prevs is None:
        X_prevs = [None] * len(As)
    roots = []
    for A, Xp in zip(As, X_prevs):
        A = A.to(torch.float64)
        if Xp is not None:
            Xp = Xp.to(torch.float64)
            Ab = dense.mm(Xp, dense.mm(A, Xp), ta=True)
            roots.append((0.5 * (Ab + Ab.T), Xp))
        else:
            roots.append((A, None))
    m = max(a.shape[0] for a, _ in roots)
    m += m & 1
    w32, V32 = _jacobi(_padded([a for a, _ in roots], m), True, 12, 1e-5)
    w32, V32 = _sort(w32, V32.to(torch.float64))
    # (root, matrix, its columns' basis in the root's space or None, ascending
    # spectrum estimate, vectors of the estimate in the matrix's space)
    todo = []
    for r, (a, B) in enumerate(roots):
        n = a.shape[0]
        V = V32[r, :n, :n]
        if n <= EXACT_BLOCK:
            V = orthonormalize(V)       # FP32-orthonormal -> FP64 (parts get it from refinement)
        todo.append((r, a, B, w32[r, :n], V))
    leaves = []
    while todo:
        r, a, B, w, V = todo.pop()
        n = a.shape[0]
        if n <= EXACT_BLOCK:
            # the part in the basis V, where it is nearly diagonal
            Ap = dense.mm(V, dense.mm(a, V), ta=True)
            leaves.append((r, 0.5 * (Ap + Ap.T), V if B is None else dense.mm(B, V)))
            continue
        s = _split_point(w, n)
        _, V = refine_projector(a, V, s, steps=steps)
        for blk in (V[:, :s], V[:, s:]):
            Ab = dense.mm(blk, dense.mm(a, blk), ta=True)
            Ab = 0.5 * (Ab + Ab.T)
            d, order = torch.sort(torch.diagonal(Ab))
            I = torch.eye(Ab.shape[0], dtype=torch.float64, device=Ab.device)[:, order].contiguous()
            todo.append((r, Ab, blk if B is None else dense.mm(B, blk), d, I))
    m = max(a.shape[0] for _, a, _ in leaves)
    m += m & 1
    w64, U64 = _jacobi(_padded([a for _, a, _ in leaves], m), False, 40, None)
    parts = [([], []) for _ in As]
    for k, (r, a, B) in enumerate(leaves):
        n = a.shape[0]
        parts[r][0].append(w64[k, :n])
        parts[r][1].append(dense.mm(B, U64[k, :n, :n].contiguous()))
    return [_sort(torch.cat(wl), torch.cat(vl, dim=1)) for wl, vl in parts]


def eigh(A, X_prev=None, refine_steps=2, exact=True, check_tol=1e-10, nocc=None):
    """Ascending eigenvalues and eigenvectors of symmetric FP64 A (..., n, n).

    n <= 136: batched FP64 Jacobi (exact to rounding; the small-molecule ensemble).
    Larger n (one matrix): exact=True or no X_prev -- spectrum slicing (exact_eigh);
    otherwise refinement from X_prev (consecutive SCF iterations): with nocc, only the
    occupied-space projector is converged (checked: orthonormal, decoupled, gapped;
    else the exact route); without nocc, full refinement (checked for orthogonality,
    else the exact route)."""
    n = A.shape[-1]
    if n <= FP64_JACOBI_MAX_N:
        if X_prev is not None:
            shape = A.shape
            A3, X3 = A.reshape(-1, n, n), X_prev.reshape(-1, n, n)
            if A3.shape[0] == 1:
                A3, X3 = A3[0], X3[0]
            Ap = dense.mm(X3, dense.mm(A3, X3), ta=True)
            w, V = jacobi(Ap)
            return _sort(w.reshape(shape[:-1]), dense.mm(X3, V).reshape(shape))
        return _sort(*jacobi(A))
    if exact or X_prev is None:
        stats["exact"] += 1
        return exact_eigh(A, X_prev)
    if nocc is not None:
        scale = max(float(A.abs().amax()), 1.0)
        X = X_prev
        for _ in range(3):
            w, X, chk = refine_projector(A, X, nocc, steps=refine_steps, check=True)
            c = chk.cpu()
            if float(c[0]) <= check_tol and float(c[1]) <= check_tol * scale and float(c[2]) < 0.0:
                stats["refined"] += 1
                wo, io = torch.sort(w[:nocc])
                wv, iv = torch.sort(w[nocc:])
                return torch.cat([wo, wv]), torch.cat([X[:, :nocc][:, io], X[:, nocc:][:, iv]], dim=1)
        stats["fallback"] += 1
        return exact_eigh(A, X_prev)
    w, X = refine(A, X_prev, steps=refine_steps + 1)
    # converged when the next correction is negligible: separated pairs' quotients and
    # the orthogonality terms R/2 both below check_tol
    R, S = _rs(A, X)
    l = torch.diagonal(S) / (1.0 - torch.diagonal(R))
    delta = 2.0 * (torch.linalg.vector_norm(S - torch.diag(l)) + torch.linalg.vector_norm(A) * torch.linalg.vector_norm(R))
    E = dense.oa_correction(S, R, 0, 1, delta=delta)
    if float(E.abs().amax()) > check_tol:
        stats["fallback"] += 1
        return exact_eigh(A, X_prev)
    return _sort(w, X)
