"""Small dense FP64 algebra of the SCF on the library's kernels (csrc/dense.cu): matrix
products with any transposes (pcg_dgemm), the Ogita-Aishima correction matrix
(pcg_oa_correction), the inverse square root of the overlap by coupled Newton-Schulz
iteration, and a DIIS whose Pulay system is solved on the GPU (pcg_diis_step).

These replace the numpy.dot / linalg products and solves of
``Methods/hartree_fock.py:168-184,226-237`` and ``Methods/hf_extensions/diis.py``;
every call is asynchronous on torch's current stream, so an SCF iteration made of them
can be captured in a CUDA graph.
"""
import ctypes
import math

import torch

from . import _lib


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def _s():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _mat(t, trans):
    """(rows, cols, row stride, col stride, batch stride) of a 2-D / 3-D tensor as op(t)."""
    sb = t.stride(0) if t.dim() == 3 else 0
    r, c = t.shape[-2], t.shape[-1]
    sr, sc = t.stride(-2), t.stride(-1)
    return (c, r, sc, sr, sb) if trans else (r, c, sr, sc, sb)


def mm(A, B, ta=False, tb=False, out=None, alpha=1.0, beta=0.0):
    """out = alpha op(A) op(B) + beta out for FP64 CUDA tensors (2-D, or 3-D batched with
    the same batch), op = transpose when ta / tb."""
    M, K, sAm, sAk, sAb = _mat(A, ta)
    K2, N, sBk, sBn, sBb = _mat(B, tb)
    if K != K2:
        raise ValueError("mm: inner dimensions differ (%d, %d)" % (K, K2))
    batch = A.shape[0] if A.dim() == 3 else (B.shape[0] if B.dim() == 3 else 1)
    if out is None:
        shape = (batch, M, N) if (A.dim() == 3 or B.dim() == 3) else (M, N)
        out = torch.empty(shape, dtype=torch.float64, device=A.device)
        beta = 0.0
    sCb = out.stride(0) if out.dim() == 3 else 0
    _lib.call("pcg_dgemm", batch, M, N, K, float(alpha), _p(A), sAb, sAm, sAk, _p(B), sBb, sBk, sBn, float(beta),
              _p(out), sCb, out.stride(-2), out.stride(-1), _s())
    return out


def oa_correction(S, R, nocc, mode, delta=None, E=None, lam=None):
    """E of one Ogita-Aishima step; delta: a 0-dim device tensor (mode 1) or None."""
    n = S.shape[0]
    E = torch.empty_like(S) if E is None else E
    _lib.call("pcg_oa_correction", n, nocc, mode, _p(delta) if delta is not None else None, _p(S), _p(R), _p(E),
              _p(lam) if lam is not None else None, _s())
    return E


def inv_sqrt(S, max_iter=60, tol=1e-13):
    """S^{-1/2} of a symmetric positive definite S by the coupled Newton-Schulz
    iteration Y <- Y T, Z <- T Z, T = (3 I - Z Y) / 2 from Y = S / c, Z = I (c = the
    Frobenius norm, so the spectrum of S / c lies in (0, 1]); quadratic convergence.
    Returns (X, ok): ok is False when the iteration did not reach ||I - Z Y|| < tol
    (a nearly singular S), and X is then not usable."""
    n = S.shape[0]
    dev = S.device
    I = torch.eye(n, dtype=torch.float64, device=dev)
    c = float(torch.linalg.vector_norm(S))
    Y = S / c
    Z = I.clone()
    ok = False
    for it in range(max_iter):
        T = mm(Z, Y, alpha=-0.5)
        T += 1.5 * I
        Y = mm(Y, T)
        Z = mm(T, Z)
        if it % 4 == 3 or it == max_iter - 1:
            err = float((mm(Z, Y) - I).abs().amax())
            if err < tol:
                ok = True
                break
    return Z / math.sqrt(c), ok


class DeviceDIIS:
    """Pulay DIIS with its state on the GPU: a ring of `cap` Fock matrices and
    residuals, the residual inner-product matrix, and the C1 solve (pcg_diis_step)."""

    def __init__(self, shape, cap, device):
        self.len = 1
        for d in shape:
            self.len *= d
        self.cap = cap
        self.state = torch.zeros(1, dtype=torch.int32, device=device)
        self.focks = torch.zeros((cap,) + tuple(shape), dtype=torch.float64, device=device)
        self.resids = torch.zeros_like(self.focks)
        self.Bm = torch.zeros(cap, cap, dtype=torch.float64, device=device)
        self.row = torch.zeros(cap, dtype=torch.float64, device=device)
        self.coef = torch.zeros(cap, dtype=torch.float64, device=device)

    def step(self, F, R, Fx):
        """Store (F, R), solve, write the extrapolated Fock matrix into Fx."""
        _lib.call("pcg_diis_step", self.len, self.cap, _p(self.state), _p(F), _p(R), _p(self.focks), _p(self.resids),
                  _p(self.Bm), _p(self.row), _p(self.coef), _p(Fx), _s())
        return Fx
