"""Closed-shell SCF and MP2 on the GPU.

Mirrors the upstream flow (``Methods/hartree_fock.py:23-154``): nuclear repulsion,
core and overlap matrices, canonical orthogonalisation X = U s^{-1/2} with
eigenvalues sorted descending and s <= 1e-6 dropped (``hartree_fock.py:226-237``),
core guess (``hartree_fock.py:55-57``), then iterations of Fock build, Pulay DIIS on
the residual X^T(SDF - FDS)X (``Methods/hf_extensions/diis.py:48-139``),
diagonalisation of X^T F X and the occupied-orbital density
(``hartree_fock.py:168-184``).

Differences kept deliberately (they change no converged energy): the energy of
iteration k is evaluated with the Fock matrix of the same density (upstream uses the
DIIS-extrapolated matrix, ``hartree_fock.py:105-108,131-133``, which is
non-variational and lets its loop report energies of diverged runs), and convergence
needs both |dE| < ``e_tol`` and RMS(dD) < ``d_tol`` (upstream: |dE| < 1e-7 only).

MP2 is the closed-shell form of ``Methods/mp2.py:43-94`` (identical value for RHF).
"""
import math
import time

import numpy as np
import torch

from . import eigen

LINEAR_DEPENDENCE = 1.0e-6   # Data/constants.py:34


def orthogonaliser(S):
    s, U = eigen.eigh(S, exact=True)
    s = torch.flip(s, [0])
    U = torch.flip(U, [1])
    keep = s > LINEAR_DEPENDENCE
    return U[:, keep] * s[keep].rsqrt()


def diis_coefficients(B):
    """Pulay C1 coefficients from the (m x m) residual inner-product matrix
    (``Methods/hf_extensions/diis.py:108-112``), solved on the host (m <= ~16)."""
    return diis_coefficients_batched(np.asarray(B)[None])[0]


def diis_coefficients_batched(Bm):
    """diis_coefficients for a stack (batch, m, m).  Each B is scaled by its largest
    diagonal entry (the coefficients do not change); a system that is still singular
    (residuals that vanished or repeat once an SCF has converged) takes the
    least-squares solution."""
    nb, m, _ = Bm.shape
    scale = np.abs(np.diagonal(Bm, axis1=1, axis2=2)).max(axis=1)
    scale = np.where(scale > 0, scale, 1.0)
    M = -np.ones((nb, m + 1, m + 1))
    M[:, :m, :m] = Bm / scale[:, None, None]
    M[:, m, m] = 0.0
    rhs = np.zeros((nb, m + 1))
    rhs[:, m] = -1.0
    try:
        return np.linalg.solve(M, rhs[..., None])[:, :m, 0]
    except np.linalg.LinAlgError:
        out = np.empty((nb, m))
        for b in range(nb):
            try:
                out[b] = np.linalg.solve(M[b], rhs[b])[:m]
            except np.linalg.LinAlgError:
                out[b] = np.linalg.lstsq(M[b], rhs[b], rcond=None)[0][:m]
        return out


class SCFResult(dict):
    __getattr__ = dict.get


def rhf(engine, max_iter=128, e_tol=1e-10, d_tol=1e-8, diis_size=10, diis_start=1, D0=None, record=False,
        guess="sad", exact_iters=3):
    """Restricted Hartree-Fock on a prepared GpuEngine.  Returns SCFResult with
    E (total), E_elec, C, eps, D (alpha density), iterations, converged.
    guess: "sad" (superposition of atomic densities, default), "core" (upstream's
    core-Hamiltonian guess), or an explicit alpha density D0.

    Fock matrices are kept in the orthonormal basis, F' = X^T F X; the DIIS residual
    is D'F' - F'D' (= X^T (S D F - F D S) X for D = X D' X^T) and DIIS extrapolates F'.
    The first exact_iters iterations diagonalise exactly; later ones refine the
    previous eigenvectors (checked, with fallback to the exact solver)."""
    mol = engine.mol
    nocc = mol.NAlphaElectrons
    if mol.NAlphaElectrons != mol.NBetaElectrons:
        raise ValueError("rhf needs a closed-shell molecule")
    S, H = engine.S, engine.H
    dev = S.device
    e_nuc = mol.nuclear_repulsion()
    X = orthogonaliser(S)
    Xt = X.T.contiguous()
    state = {"Q": None}

    def diagonalise(Fp, exact=False):
        e, Q = eigen.eigh(Fp, X_prev=state["Q"], refine_steps=2, exact=exact, nocc=nocc)
        state["Q"] = Q
        return e, X @ Q

    if D0 is not None:
        D = D0.clone()
    elif guess == "sad":
        from .guess import sad_density
        D = sad_density(mol, device=dev)
    else:
        eps, C = diagonalise(Xt @ H @ X)
        D = C[:, :nocc] @ C[:, :nocc].T
    Dp = Xt @ S @ D @ S @ X      # orthonormal-basis density
    n = engine.nbf
    F = torch.empty(n, n, dtype=torch.float64, device=dev)
    G = torch.empty(n, n, dtype=torch.float64, device=dev)
    focks, resids = [], []
    Bmat = np.zeros((0, 0))
    E_old = D_old = None
    history = []
    converged = False
    it = 0
    for it in range(1, max_iter + 1):
        engine.fock(D, out=F, G=G)
        use_diis = it > diis_start
        Fp = Xt @ F @ X
        if use_diis:
            P = Dp @ Fp
            R = P - P.T
        else:
            R = None
        # one device->host read per iteration: energy, density change, new DIIS row
        vals = [torch.sum(D * (H + F)).reshape(1)]
        vals.append(torch.sqrt(torch.mean((D - D_old) ** 2)).reshape(1) if D_old is not None
                    else torch.zeros(1, dtype=torch.float64, device=dev))
        if use_diis:
            rv = R.reshape(-1)
            vals.append(torch.stack([torch.dot(rv, r.reshape(-1)) for r in resids] + [torch.dot(rv, rv)]))
        host = torch.cat(vals).cpu().numpy()
        E = float(host[0]) + e_nuc
        if E_old is not None:
            drms = float(host[1])
            dE = E - E_old
            if record:
                history.append((it, E, dE, drms))
            if abs(dE) < e_tol and drms < d_tol:
                converged = True
                break
        E_old, D_old = E, D
        Fx = Fp
        if use_diis:
            row = host[2:]
            m = len(resids) + 1
            Bn = np.zeros((m, m))
            Bn[:m - 1, :m - 1] = Bmat
            Bn[m - 1, :] = row
            Bn[:, m - 1] = row
            focks.append(Fp)
            resids.append(R)
            Bmat = Bn
            if len(focks) > diis_size:
                focks.pop(0); resids.pop(0)
                Bmat = Bmat[1:, 1:]
            if len(focks) > 1:
                c = diis_coefficients(Bmat)
                cw = torch.tensor(c, dtype=torch.float64, device=dev)
                Fx = torch.einsum("k,kij->ij", cw, torch.stack(focks))
        eps, C = diagonalise(Fx, exact=it <= exact_iters)
        Co = C[:, :nocc]
        D = Co @ Co.T
        Qo = state["Q"][:, :nocc]
        Dp = Qo @ Qo.T
    # orbitals of the final Fock matrix, exact (including inside near-degenerate
    # clusters) for MP2's denominators
    eps, C = diagonalise(Xt @ F @ X, exact=True)
    return SCFResult(E=E, E_elec=E - e_nuc, E_nuc=e_nuc, C=C, eps=eps, D=D, F=F, iterations=it,
                     converged=converged, history=history, fock_builds=it)


def ozaki_gemm(A, B, C, batch, M, N, K, sA, sB, sCb, nslice=6, accumulate=False):
    """C[b][m][n] (+)= sum_k A[b,m,k] B[b,k,n] in FP64 accuracy on BF16 tensor cores
    (pcg_ozaki_gemm); sA = (sAb, sAm, sAk), sB = (sBb, sBk, sBn) element strides."""
    import ctypes
    from . import _lib
    d = _lib.GemmDescT(batch, M, N, K, sA[0], sA[1], sA[2], sB[0], sB[2], sB[1], sCb)
    nbytes = _lib.load().pcg_ozaki_workspace(ctypes.byref(d), nslice)
    ws = torch.empty(nbytes, dtype=torch.uint8, device=C.device)
    _lib.call("pcg_ozaki_gemm", ctypes.byref(d), ctypes.c_void_p(A.data_ptr()), ctypes.c_void_p(B.data_ptr()),
              ctypes.c_void_p(C.data_ptr()), nslice, 1 if accumulate else 0, ctypes.c_void_p(ws.data_ptr()), nbytes,
              ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    return C


def mp2_transform(eri, Co, Cv, gemm="ozaki", nslice=6):
    """(ia|jb) from the dense AO tensor by four quarter transforms.
    gemm="fp64": cuBLAS DGEMM; gemm="ozaki": BF16 tensor cores with FP64 accuracy."""
    n, o = Co.shape
    v = Cv.shape[1]
    if gemm == "fp64":
        t1 = (Co.T @ eri.reshape(n, n ** 3)).reshape(o, n, n * n)        # (i nu | lam sig)
        t2 = torch.matmul(Cv.T, t1)                                       # (i a | lam sig)
        del t1
        t3 = torch.matmul(Co.T, t2.reshape(o * v, n, n))                  # (i a | j sig)
        del t2
        return torch.matmul(t3, Cv).reshape(o, v, o, v)                   # (i a | j b)
    dev = eri.device
    E = eri.reshape(-1)
    Co, Cv = Co.contiguous(), Cv.contiguous()
    # Y1[i][(b c d)] = sum_a Co[a][i] E[a][(b c d)]
    Y1 = torch.empty(o * n ** 3, dtype=torch.float64, device=dev)
    ozaki_gemm(Co, E, Y1, 1, o, n ** 3, n, (0, 1, o), (0, n ** 3, 1), 0, nslice)
    # Y2[i][a'][(c d)] = sum_b Cv[b][a'] Y1[i][b][(c d)]
    Y2 = torch.empty(o * v * n * n, dtype=torch.float64, device=dev)
    ozaki_gemm(Cv, Y1, Y2, o, v, n * n, n, (0, 1, v), (n ** 3, n * n, 1), v * n * n, nslice)
    del Y1
    # Y3[(i a)][j][d] = sum_c Co[c][j] Y2[(i a)][c][d]
    Y3 = torch.empty(o * v * o * n, dtype=torch.float64, device=dev)
    ozaki_gemm(Co, Y2, Y3, o * v, o, n, n, (0, 1, o), (n * n, n, 1), o * n, nslice)
    del Y2
    # T[(i a j)][b] = sum_d Y3[(i a j)][d] Cv[d][b]
    T = torch.empty(o * v * o * v, dtype=torch.float64, device=dev)
    ozaki_gemm(Y3, Cv, T, 1, o * v * o, v, n, (0, n, 1), (0, v, 1), 0, nslice)
    return T.reshape(o, v, o, v)


def rmp2(engine, C, eps, eri=None, gemm="ozaki", nslice=6):
    """Closed-shell MP2 correlation energy: four quarter transforms of the dense AO
    tensor to (ia|jb) and the energy denominator sum."""
    mol = engine.mol
    o = mol.NAlphaElectrons
    if eri is None:
        eri = engine.dense_eri()
    Co = C[:, :o].contiguous()
    Cv = C[:, o:].contiguous()
    ovov = mp2_transform(eri, Co, Cv, gemm=gemm, nslice=nslice)
    eo, ev = eps[:o], eps[o:]
    den = eo[:, None, None, None] - ev[None, :, None, None] + eo[None, None, :, None] - ev[None, None, None, :]
    e2 = torch.sum(ovov * (2.0 * ovov - ovov.permute(0, 3, 2, 1)) / den)
    return float(e2)


def mp2_flops(n, o, v):
    return 2.0 * o * n ** 4 + 2.0 * o * v * n ** 3 + 2.0 * o * o * v * n ** 2 + 2.0 * o * o * v * v * n
