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

import torch

LINEAR_DEPENDENCE = 1.0e-6   # Data/constants.py:34


def orthogonaliser(S):
    s, U = torch.linalg.eigh(S)
    s = torch.flip(s, [0])
    U = torch.flip(U, [1])
    keep = s > LINEAR_DEPENDENCE
    return U[:, keep] * s[keep].rsqrt()


class SCFResult(dict):
    __getattr__ = dict.get


def rhf(engine, max_iter=128, e_tol=1e-10, d_tol=1e-8, diis_size=10, diis_start=1, D0=None, record=False):
    """Restricted Hartree-Fock on a prepared GpuEngine.  Returns SCFResult with
    E (total), E_elec, C, eps, D (alpha density), iterations, converged, timings."""
    mol = engine.mol
    nocc = mol.NAlphaElectrons
    if mol.NAlphaElectrons != mol.NBetaElectrons:
        raise ValueError("rhf needs a closed-shell molecule")
    S, H = engine.S, engine.H
    e_nuc = mol.nuclear_repulsion()
    X = orthogonaliser(S)
    Xt = X.T.contiguous()

    def diagonalise(F):
        e, Cp = torch.linalg.eigh(Xt @ F @ X)
        return e, X @ Cp

    if D0 is None:
        eps, C = diagonalise(H)
        D = C[:, :nocc] @ C[:, :nocc].T
    else:
        D = D0.clone()
    n = engine.nbf
    F = torch.empty(n, n, dtype=torch.float64, device=S.device)
    G = torch.empty(n, n, dtype=torch.float64, device=S.device)
    focks, resids = [], []
    E_old = None
    history = []
    converged = False
    it = 0
    t_fock = 0.0
    for it in range(1, max_iter + 1):
        t0 = time.perf_counter()
        engine.fock(D, out=F, G=G)
        E = float(torch.sum(D * (H + F))) + e_nuc
        t_fock += time.perf_counter() - t0
        drms = None
        if E_old is not None:
            drms = float(torch.sqrt(torch.mean((D - D_old) ** 2)))
            dE = E - E_old
            if record:
                history.append((it, E, dE, drms))
            if abs(dE) < e_tol and drms < d_tol:
                converged = True
                break
        E_old, D_old = E, D
        R = Xt @ (S @ D @ F - F @ D @ S) @ X
        Fx = F
        if it > diis_start:
            focks.append(F.clone())
            resids.append(R)
            if len(focks) > diis_size:
                focks.pop(0); resids.pop(0)
            m = len(focks)
            if m > 1:
                Rs = torch.stack([r.reshape(-1) for r in resids])
                B = torch.empty(m + 1, m + 1, dtype=torch.float64, device=S.device)
                B[:m, :m] = Rs @ Rs.T
                B[m, :m] = -1.0
                B[:m, m] = -1.0
                B[m, m] = 0.0
                rhs = torch.zeros(m + 1, dtype=torch.float64, device=S.device)
                rhs[m] = -1.0
                c = torch.linalg.solve(B, rhs)[:m]
                Fx = torch.einsum("k,kij->ij", c, torch.stack(focks))
        eps, C = diagonalise(Fx)
        D = C[:, :nocc] @ C[:, :nocc].T
    # orbitals of the final Fock matrix
    eps, C = diagonalise(F)
    return SCFResult(E=E, E_elec=E - e_nuc, E_nuc=e_nuc, C=C, eps=eps, D=D, F=F, iterations=it,
                     converged=converged, history=history, fock_builds=it, t_fock=t_fock)


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
