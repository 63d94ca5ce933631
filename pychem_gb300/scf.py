"""SCF and MP2 on the GPU: RHF (rhf), UHF / CUHF with MOM (uhf), RMP2 (rmp2), UMP2
(ump2).

Mirrors the upstream flow (``Methods/hartree_fock.py:23-154``): nuclear repulsion,
core and overlap matrices, an orthogonaliser X (upstream's canonical U s^{-1/2} with
s <= 1e-6 dropped, ``hartree_fock.py:226-237``, or a Cholesky factor when no
eigenvalue is near that cut), a starting density (SAD by default; upstream's core
guess, ``hartree_fock.py:55-57``, on request), then iterations of Fock build, Pulay
DIIS on the residual X^T(SDF - FDS)X (``Methods/hf_extensions/diis.py:48-139``),
diagonalisation of X^T F X and the occupied-orbital density
(``hartree_fock.py:168-184``).

Differences kept deliberately (they change no converged energy): the energy of
iteration k is evaluated with the Fock matrix of the same density (upstream uses the
DIIS-extrapolated matrix, ``hartree_fock.py:105-108,131-133``, which is
non-variational and lets its loop report energies of diverged runs), and convergence
needs both |dE| < ``e_tol`` and RMS(dD) < ``d_tol`` (upstream: |dE| < 1e-7 only).

RMP2 is the closed-shell form of ``Methods/mp2.py:43-94`` (identical value for RHF);
the AO->MO transforms run on the tcgen05 tensor cores with FP64 accuracy
(ozaki_gemm_tc: Ozaki digit slices, every level in one kernel).
"""
import ctypes
import math
import time

import numpy as np
import torch

from . import _lib, eigen

LINEAR_DEPENDENCE = 1.0e-6   # Data/constants.py:34


def orthogonaliser(S, canonical=False):
    """X with X^T S X = I.  Upstream (hartree_fock.py:226-237) uses the canonical
    U s^-1/2 with eigenvalues s <= 1e-6 dropped.  For n > 136, unless canonical=True,
    the symmetric X = S^-1/2 from the coupled Newton-Schulz iteration (library GEMMs
    only) is used when the smallest eigenvalue of S, estimated by power iteration on
    X^2 = S^-1, is above 1e-5: then nothing would be dropped and energies and orbitals
    do not depend on the choice of X; otherwise the canonical route."""
    from . import dense
    n = S.shape[0]
    if not canonical and n > eigen.FP64_JACOBI_MAX_N:
        X, ok = dense.inv_sqrt(S)
        if ok:
            # power iteration on X^2 = S^-1, on the device; the host reads the result once
            v = torch.ones(n, 1, dtype=S.dtype, device=S.device) / math.sqrt(n)
            for _ in range(16):
                w = dense.mm(X, dense.mm(X, v))
                nrm = torch.linalg.vector_norm(w)
                v = w / nrm
            mu = float(nrm)
            if 1.0 / mu > 10.0 * LINEAR_DEPENDENCE:
                return X
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
        guess="sad", exact_iters=1, graph=None):
    """Restricted Hartree-Fock on a prepared GpuEngine.  Returns SCFResult with
    E (total), E_elec, C, eps, D (alpha density), iterations, converged.
    guess: "sad" (superposition of atomic densities, default), "core" (upstream's
    core-Hamiltonian guess), or an explicit alpha density D0.

    Fock matrices are kept in the orthonormal basis, F' = X^T F X; the DIIS residual
    is D'F' - F'D' (= X^T (S D F - F D S) X for D = X D' X^T) and DIIS extrapolates F'
    with its Pulay system solved on the GPU.  Every step runs on the library's
    kernels: Fock digestion, FP64 GEMMs (pcg_dgemm), the eigenvectors (Jacobi for the
    first exact_iters iterations, then refinement of the previous vectors that
    decouples the occupied space, checked, with the Jacobi route when the check
    fails), the density C_occ C_occ^T on the tensor cores (pcg_ozaki_gemm_tc).  For
    n > 136 (graph None or True) every iteration after the first exact_iters is one
    CUDA graph replay followed by one read of six numbers (energy, density change,
    refinement checks, commutator size)."""
    from . import dense
    mol = engine.mol
    nocc = mol.NAlphaElectrons
    if mol.NAlphaElectrons != mol.NBetaElectrons:
        raise ValueError("rhf needs a closed-shell molecule")
    S, H = engine.S, engine.H
    dev = S.device
    e_nuc = mol.nuclear_repulsion()
    n = engine.nbf
    big = n > eigen.FP64_JACOBI_MAX_N
    use_graph = big if graph is None else (graph and big)
    X = orthogonaliser(S)
    n2 = X.shape[1]
    mm = dense.mm

    # static buffers (the CUDA graph reads and writes these addresses)
    D = torch.empty(n, n, dtype=torch.float64, device=dev)
    if D0 is not None:
        D.copy_(D0)
    elif guess == "sad":
        from .guess import sad_density
        D.copy_(sad_density(mol, device=dev))
    else:
        _, Q0 = eigen.eigh(mm(X, mm(H, X), ta=True), exact=True)
        C0 = mm(X, Q0)
        mm(C0[:, :nocc], C0[:, :nocc], tb=True, out=D)
    Dp = mm(X, mm(mm(S, D), mm(S, X)), ta=True)      # orthonormal-basis density
    F = torch.empty(n, n, dtype=torch.float64, device=dev)
    G = torch.empty(n, n, dtype=torch.float64, device=dev)
    Fp = torch.empty(n2, n2, dtype=torch.float64, device=dev)
    R = torch.empty(n2, n2, dtype=torch.float64, device=dev)
    Fx = torch.empty(n2, n2, dtype=torch.float64, device=dev)
    Q = torch.eye(n2, dtype=torch.float64, device=dev)
    C = torch.empty(n, n2, dtype=torch.float64, device=dev)
    Dold = torch.zeros(n, n, dtype=torch.float64, device=dev)
    vals = torch.zeros(6, dtype=torch.float64, device=dev)
    diis = dense.DeviceDIIS((n2, n2), diis_size, dev)
    have_q = [False]

    def fock_and_diis(use_diis):
        engine.fock(D, out=F, G=G)
        mm(X, mm(F, X), ta=True, out=Fp)
        P = mm(Dp, Fp)
        torch.sub(P, P.T, out=R)
        vals[0] = torch.sum(D * (H + F))
        vals[1] = torch.sqrt(torch.mean((D - Dold) ** 2))
        vals[5] = R.abs().amax()
        Dold.copy_(D)
        if use_diis:
            diis.step(Fp, R, Fx)
        else:
            Fx.copy_(Fp)

    def density():
        mm(X, Q, out=C)
        if big:
            ozaki_gemm_tc(C, C, D, n, n, nocc, n2, (1, n2), (n, 1))      # D = C_occ C_occ^T
        else:
            mm(C[:, :nocc], C[:, :nocc], tb=True, out=D)
        mm(Q[:, :nocc], Q[:, :nocc], tb=True, out=Dp)

    def diag_exact():
        if big:
            # a few FP32 Jacobi sweeps put the occupied space well inside the HOMO-LUMO
            # gap; the projector refinement does the rest in FP64
            _, V = eigen.eigh32_own(Fx, Q if have_q[0] else None, tol=1e-4, max_sweeps=5)
            _, V = eigen.refine_projector(Fx, V, nocc, steps=3)
        else:
            _, V = eigen.eigh(Fx, X_prev=Q if have_q[0] else None)
        Q.copy_(V)
        have_q[0] = True
        vals[2:5] = 0.0

    def diag_refine():
        _, V, chk = eigen.refine_projector(Fx, Q, nocc, steps=2, check=True)
        Q.copy_(V)
        vals[2:5] = chk

    g = None
    per_replay = 0
    E_old = None
    history = []
    phases = {}
    if record:
        torch.cuda.synchronize()
        phases["setup"] = time.perf_counter()
    fallbacks = 0
    t_last = time.perf_counter()
    converged = False
    it = 0
    scale = None
    for it in range(1, max_iter + 1):
        exact = it <= exact_iters or not big
        if exact or not use_graph:
            fock_and_diis(it > diis_start)
            if exact:
                diag_exact()
            else:
                diag_refine()
            density()
        else:
            if g is None:
                torch.cuda.synchronize()
                g = torch.cuda.CUDAGraph()
                c0 = _lib_launches()
                # captured on a side stream with the graph pool, without the
                # torch.cuda.graph context's gc.collect() and empty_cache() (which
                # would hand the allocator's cached blocks back to the driver)
                side, pool = _graph_stream_and_pool(dev)
                side.wait_stream(torch.cuda.current_stream())
                with torch.cuda.stream(side):
                    g.capture_begin(pool=pool)
                    try:
                        fock_and_diis(True)
                        diag_refine()
                        density()
                    finally:
                        g.capture_end()
                torch.cuda.current_stream().wait_stream(side)
                # keeps the pool alive (its use count) until the next solve's capture;
                # the graph it replaces returns its blocks to the pool
                _LAST_GRAPH[dev] = g
                per_replay = _lib_launches() - c0
                if record:
                    phases["capture"] = time.perf_counter()
            g.replay()
            _lib_add_launches(per_replay)
        host = vals.cpu().numpy()
        if record and it <= 2:
            phases["iteration%d" % it] = time.perf_counter()
        E = float(host[0]) + e_nuc
        if not exact:
            if scale is None:
                scale = max(float(Fx.abs().amax()), 1.0)
            # the refined occupied space need only be as good as the SCF itself: Q stays
            # orthonormal, so D is a valid (idempotent) density, and its coupling to the
            # virtual space must be small against this iteration's commutator; near
            # convergence that means fully refined
            ov_tol = max(1e-10 * scale, 0.1 * float(host[5]))
            ok = host[2] <= 1e-10 and host[3] <= ov_tol and host[4] < 0.0
            if not ok:
                # refinement not yet converged (a large step early on): more steps from
                # where it stopped, then the Jacobi route
                fallbacks += 1
                for _ in range(4):
                    _, V, chk = eigen.refine_projector(Fx, Q, nocc, steps=3, check=True, ortho_steps=2)
                    Q.copy_(V)
                    c = chk.cpu().numpy()
                    if c[0] <= 1e-10 and c[1] <= ov_tol and c[2] < 0.0:
                        ok = True
                        break
                if not ok:
                    diag_exact()
                density()
        if E_old is not None:
            drms = float(host[1])
            dE = E - E_old
            if record:
                now = time.perf_counter()
                history.append((it, E, dE, drms, now - t_last, tuple(float(x) for x in host[2:5])))
                t_last = now
            if abs(dE) < e_tol and drms < d_tol:
                converged = True
                break
        E_old = E
    # orbitals of the final Fock matrix, exact (including inside near-degenerate
    # clusters) for MP2's denominators: for n > 136 the occupied and virtual blocks of
    # the refined vectors are decoupled once more and each block is diagonalised
    # exactly (spectrum slicing inside blocks above 136)
    if record:
        torch.cuda.synchronize()
        phases["loop"] = time.perf_counter()
    Ff = mm(X, mm(F, X), ta=True)
    if big:
        _, V = eigen.refine_projector(Ff, Q, nocc, steps=2)
        blks = (V[:, :nocc], V[:, nocc:])
        Abs = [mm(blk, mm(Ff, blk), ta=True) for blk in blks]
        res = eigen.exact_eigh_many([0.5 * (Ab + Ab.T) for Ab in Abs])
        eps = torch.cat([wb for wb, _ in res])
        Qf = torch.cat([mm(blk, Ub) for blk, (_, Ub) in zip(blks, res)], dim=1)
    else:
        eps, Qf = eigen.eigh(Ff, exact=True)
    Cf = mm(X, Qf)
    Dn = mm(Cf[:, :nocc], Cf[:, :nocc], tb=True)
    if record:
        torch.cuda.synchronize()
        phases["final"] = time.perf_counter()
    return SCFResult(phases=phases, E=E, E_elec=E - e_nuc, E_nuc=e_nuc, C=Cf, eps=eps, D=Dn, F=F, iterations=it,
                     converged=converged, history=history, fock_builds=it, diag_fallbacks=fallbacks)


_GRAPH_POOLS = {}
_LAST_GRAPH = {}


def _graph_stream_and_pool(dev):
    """A capture stream and one memory pool per device for the SCF iteration graphs:
    a new solve's capture takes its buffers from the pool, where the graph before the
    previous one left them (the previous graph is kept, never replayed again, until
    the capture that replaces it, so that the pool stays in use)."""
    if dev not in _GRAPH_POOLS:
        with torch.cuda.device(dev):
            _GRAPH_POOLS[dev] = (torch.cuda.Stream(), torch.cuda.graph_pool_handle())
    return _GRAPH_POOLS[dev]


def _lib_launches():
    from . import _lib
    return _lib.launch_count


def _lib_add_launches(k):
    from . import _lib
    _lib.launch_count += k


_TC_WS = {}


def _tc_workspace(dev, nbytes):
    """A cached device workspace for pcg_ozaki_gemm_tc (grown on demand)."""
    ws = _TC_WS.get(dev)
    if ws is None or ws.numel() < nbytes:
        ws = torch.empty(max(nbytes, 1 << 20), dtype=torch.uint8, device=dev)
        _TC_WS[dev] = ws
    return ws


def ozaki_gemm_tc(X, Y, C, M, N, K, ldx, sY, sC, nslice=6, accumulate=False):
    """C[m*sC[0] + n*sC[1]] (+)= sum_k X[m*ldx + k] Y[k*sY[0] + n*sY[1]] in FP64 accuracy
    with every Ozaki level in one tcgen05 tensor-core kernel (pcg_ozaki_gemm_tc); X is
    split into BF16 digit slices on the fly.  Element offsets are relative to the
    tensors' data pointers."""
    import ctypes
    from . import _lib
    lib = _lib.load()
    nbytes = lib.pcg_ozaki_tc_workspace(N, K, nslice)
    ws = _tc_workspace(C.device, nbytes)
    _lib.call("pcg_ozaki_gemm_tc", M, N, K, ctypes.c_void_p(X.data_ptr()), ldx, ctypes.c_void_p(Y.data_ptr()),
              sY[0], sY[1], ctypes.c_void_p(C.data_ptr()), sC[0], sC[1], nslice, 1 if accumulate else 0,
              ctypes.c_void_p(ws.data_ptr()), ws.numel(), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    return C


def ozaki_tc_status(dev):
    """Error flag of the last pcg_ozaki_gemm_tc on this device (0 = every wait ended)."""
    import ctypes
    from . import _lib
    ws = _TC_WS.get(torch.device(dev) if not isinstance(dev, torch.device) else dev)
    if ws is None:
        return 0
    return _lib.load().pcg_ozaki_tc_status(ctypes.c_void_p(ws.data_ptr()),
                                           ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))


def _pair_rows(n, dev):
    """Row index a*n + b of every AO pair a >= b in pair order (pair(a, b) = a(a+1)/2 + b)."""
    a, b = torch.tril_indices(n, n, device=dev)
    return a * n + b


def mp2_transform(eri, Co, Cv, gemm="tc", nslice=6, Co2=None, Cv2=None, timings=None):
    """(ia|jb) from the AO integrals by four quarter transforms, i, a with Co, Cv and
    j, b with Co2, Cv2 (default: the same; different for the opposite-spin block of
    UMP2).  eri: the dense tensor (n, n, n, n), the bra-pair-packed one
    (n(n+1)/2, n, n) of GpuEngine.dense_eri_pairs, or its compact form (E, map, rows)
    (dense_eri_pairs(compact=True): only the AO pairs some stored quartet contains, so
    the first two transforms skip the rows that screening leaves zero).

    gemm="tc": each transform is one pcg_ozaki_gemm_tc launch (FP64-accurate on the
    tcgen05 tensor cores) contracting the last, contiguous index of its input and
    writing its output transposed, so that the next transform again contracts a
    contiguous index; the first two keep the bra pair packed (ab) = (ba):
        T1[i][ab c] = sum_d (ab|cd) Co[d][i]          T2[a'][i ab] = sum_c T1 Cv[c][a']
        T2 unpacked to [a'][i][a][b]                   T3[j][a' i a] = sum_b T2 Co2[b][j]
        T4[b'][j a' i] = sum_a T3 Cv2[a][b']           T4[b'][j][a'][i] = (i a'|j b').
    gemm="fp64": the same contraction by FP64 matrix products on the dense tensor
    (cuBLAS DGEMM through torch), the cross-check.  timings (a list) receives
    (M, N, K, (start, end) CUDA events) of every tensor-core launch."""
    n, o = Co.shape
    v = Cv.shape[1]
    Co2 = Co if Co2 is None else Co2
    Cv2 = Cv if Cv2 is None else Cv2
    o2, v2 = Co2.shape[1], Cv2.shape[1]
    npair = n * (n + 1) // 2
    if gemm == "fp64":
        if eri.dim() != 4:
            raise ValueError("gemm='fp64' needs the dense (n, n, n, n) tensor")
        t1 = (Co.T @ eri.reshape(n, n ** 3)).reshape(o, n, n * n)        # (i nu | lam sig)
        t2 = torch.matmul(Cv.T, t1)                                       # (i a | lam sig)
        del t1
        t3 = torch.matmul(Co2.T, t2.reshape(o * v, n, n))                 # (i a | j sig)
        del t2
        return torch.matmul(t3, Cv2).reshape(o, v, o2, v2)                # (i a | j b)
    if gemm != "tc":
        raise ValueError("gemm must be 'tc' or 'fp64'")
    import ctypes
    from . import _lib
    pmap = None
    if isinstance(eri, tuple):                       # (E, map, rows) of dense_eri_pairs(compact=True)
        eri, pmap, npair = eri
    dev = eri.device
    if eri.dim() == 4:
        eri = eri.reshape(n * n, n * n)[_pair_rows(n, dev)]
    E = eri.reshape(-1)
    Co, Cv, Co2, Cv2 = Co.contiguous(), Cv.contiguous(), Co2.contiguous(), Cv2.contiguous()

    def quarter(X, rows, C, ncol):
        out = torch.empty(ncol * rows, dtype=torch.float64, device=dev)
        if timings is not None:
            ev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
            ev[0].record()
        ozaki_gemm_tc(X, C, out, rows, ncol, n, n, (ncol, 1), (1, rows), nslice=nslice)
        if timings is not None:
            ev[1].record()
            timings.append((rows, ncol, n, ev))
        return out

    T1 = quarter(E, npair * n, Co, o)
    T2p = quarter(T1, o * npair, Cv, v)
    del T1
    T2 = torch.empty(v * o * n * n, dtype=torch.float64, device=dev)
    from .engine import pair_colmap
    cm = pair_colmap(n, pmap, dev)
    _lib.call("pcg_unpack_pairs", v * o, n, npair, ctypes.c_void_p(cm.data_ptr()), ctypes.c_void_p(T2p.data_ptr()),
              ctypes.c_void_p(T2.data_ptr()), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    del T2p
    T3 = quarter(T2, v * o * n, Co2, o2)
    del T2
    T4 = quarter(T3, o2 * v * o, Cv2, v2)
    return T4.view(v2, o2, v, o).permute(3, 2, 1, 0)


MP2_SCALES = {"MP2": None, "MP2-SCS": (1.0 / 3.0, 6.0 / 5.0), "MP2-SOS": (0.0, 1.3)}   # Methods/mp2.py:97-107


def rmp2(engine, C, eps, eri=None, gemm="tc", nslice=6, scale=None):
    """Closed-shell MP2 correlation energy: four quarter transforms of the dense AO
    tensor to (ia|jb) and the energy denominator sum.  scale = (c_ss, c_os) weights
    the same-spin part sum (ia|jb)((ia|jb) - (ib|ja))/D and the opposite-spin part
    sum (ia|jb)^2/D (MP2_SCALES: SCS and SOS as Methods/mp2.py:97-107)."""
    mol = engine.mol
    o = mol.NAlphaElectrons
    if eri is None:
        eri = engine.dense_eri() if gemm == "fp64" else engine.dense_eri_pairs(compact=True)
    Co = C[:, :o].contiguous()
    Cv = C[:, o:].contiguous()
    ovov = mp2_transform(eri, Co, Cv, gemm=gemm, nslice=nslice)
    s1, s2 = mp2_pair_sums(ovov, eps[:o].contiguous(), eps[o:].contiguous())
    if scale is not None:
        return scale[0] * (s1 - s2) + scale[1] * s1        # same spin, opposite spin
    return 2.0 * s1 - s2


def mp2_pair_sums(ovov, eo, ev):
    """(s1, s2) = (sum (ia|jb)^2 / D, sum (ia|jb)(ib|ja) / D), D = e_i + e_j - e_a - e_b,
    in one kernel (pcg_mp2_pair_sums) over ovov[i, a, j, b] stored b-major (the layout
    mp2_transform returns)."""
    o, v = ovov.shape[0], ovov.shape[1]
    X = ovov.permute(3, 2, 1, 0)
    if not X.is_contiguous() or ovov.shape[2] != o or ovov.shape[3] != v:
        X = ovov.permute(3, 2, 1, 0).contiguous()
    part = torch.empty(o * v, 2, dtype=torch.float64, device=ovov.device)
    vp = ctypes.c_void_p
    _lib.call("pcg_mp2_pair_sums", o, v, vp(X.data_ptr()), vp(eo.data_ptr()), vp(ev.data_ptr()), vp(part.data_ptr()),
              vp(torch.cuda.current_stream().cuda_stream))
    s = part.sum(0).tolist()
    return s[0], s[1]


def mp2_flops(n, o, v):
    return 2.0 * o * n ** 4 + 2.0 * o * v * n ** 3 + 2.0 * o * o * v * n ** 2 + 2.0 * o * o * v * v * n


# ------------------------------------------------------------------------------------
# Open shells: UHF / CUHF and UMP2
# ------------------------------------------------------------------------------------
class _SpinDIIS:
    """Per-spin Pulay DIIS as Methods/hf_extensions/diis.py:14-154: a residual enters
    the space only while its largest element is below 0.5, C1 coefficients solved on
    the host, the oldest vectors dropped while the B matrix's eigenvalue condition
    number exceeds 1e7; the extrapolation runs on the GPU."""

    def __init__(self):
        self.res, self.focks = [], []
        self.B = np.zeros((0, 0))

    def extrapolate(self, R, F, row, rmax):
        """R, F: this iteration's residual and Fock (device); row: inner products of R
        with the stored residuals and itself (host); rmax: max element of R."""
        if not abs(rmax) < 0.5:
            return F, False
        m = len(self.res) + 1
        Bn = np.zeros((m, m))
        Bn[:m - 1, :m - 1] = self.B
        Bn[m - 1, :] = row
        Bn[:, m - 1] = row
        self.B = Bn
        self.res.append(R)
        self.focks.append(F)
        if m < 2:
            return F, True
        while True:
            m = len(self.res)
            M = -np.ones((m + 1, m + 1))
            M[:m, :m] = self.B
            M[m, m] = 0.0
            ev = np.abs(np.linalg.eigvals(M))
            if (ev.min() > 0 and ev.max() / ev.min() <= 1e7) or m == 1:
                break
            self.res.pop(0); self.focks.pop(0)
            self.B = self.B[1:, 1:]
        rhs = np.zeros(m + 1)
        rhs[m] = -1.0
        c = np.linalg.solve(M, rhs)[:m]
        cw = torch.tensor(c, dtype=torch.float64, device=F.device)
        return torch.einsum("k,kij->ij", cw, torch.stack(self.focks)), True


def mom_order(C, e, C_ref, n, S):
    """Maximum overlap ordering (Methods/hf_extensions/mom.py:6-47): columns of C by
    decreasing |sum_j <ref_j|C_i>| over the n occupied reference orbitals."""
    p = ((C_ref[:, :n].T @ S) @ C).sum(dim=0).abs()
    order = torch.argsort(-p, stable=True)
    return C[:, order], e[order]


def _sort_occupied(C, e, n):
    """The first n columns ordered by energy, the rest kept (Util/structures.py:923-929)."""
    if n > 1:
        idx = torch.cat([torch.argsort(e[:n], stable=True), torch.arange(n, e.shape[0], device=e.device)])
        C, e = C[:, idx], e[idx]
    return C, e


def uhf(engine, cuhf=False, max_iter=300, e_tol=1e-10, d_tol=1e-8, C0=None, mom=False, occ=None,
        cuhf_spaces=None):
    """Unrestricted (cuhf=False) or constrained unrestricted Hartree-Fock on a prepared
    GpuEngine, along Methods/hartree_fock.py:23-142: core-Hamiltonian guess for both
    spins, Fock matrices from pcg_digest_class_u, the CUHF constraint of
    hartree_fock.py:359-391 (natural orbitals of S^1/2 (D_tot/2) S^1/2, the core-virtual
    block of (F_a - F_b)/2 cancelled), per-spin DIIS, aufbau occupation, energy
    0.5 sum(D_tot H + D_a F_a + D_b F_b) (hartree_fock.py:188-201) from the Fock
    matrices of the current densities.  C0 = (Ca, Cb): starting orbitals, occupied
    columns first (an excited determinant) instead of the core guess; mom: occupy by
    maximum overlap with C0's occupied orbitals (the FIXED reference of
    Methods/hf_extensions/mom.py) instead of aufbau, the occupied orbitals then sorted
    by energy (Util/structures.py:923-929).  occ = (n_alpha, n_beta) for a state other
    than the molecule's own; cuhf_spaces = (core, active) counts of the constraint
    (doubly and singly occupied positions of the state's occupancy lists,
    hartree_fock.py:361-365), default (n_beta, n_alpha - n_beta).  Returns SCFResult
    with E, Ca, Cb, ea, eb, Da, Db, iterations, converged."""
    mol = engine.mol
    na, nb = occ if occ is not None else (mol.NAlphaElectrons, mol.NBetaElectrons)
    ncore, nact = cuhf_spaces if cuhf_spaces is not None else (nb, na - nb)
    S, H = engine.S, engine.H
    dev = S.device
    e_nuc = mol.nuclear_repulsion()
    s, U = eigen.eigh(S)
    if float(s.min()) <= LINEAR_DEPENDENCE:
        raise ValueError("linear dependence in the basis; uhf needs a full-rank overlap")
    X = U * s.rsqrt().unsqueeze(0)
    Xt = X.T.contiguous()
    Sh = (U * s.sqrt().unsqueeze(0)) @ U.T          # S^1/2 (hartree_fock.py:234-237)
    Shi = X @ U.T                                   # (S^1/2)^-1

    def diag(F):
        e, Q = eigen.eigh(Xt @ F @ X)
        return e, X @ Q

    def constrain(Da, Db, Fa, Fb):
        vals, V = eigen.eigh(Sh @ (0.5 * (Da + Db)) @ Sh)
        Cno = Shi @ V
        back = V.T @ Sh                             # Cno^-1
        order = torch.argsort(vals, descending=True)
        core, virt = order[:ncore], order[ncore + nact:]
        delta = Cno.T @ (0.5 * (Fa - Fb)) @ Cno
        lam = torch.zeros_like(delta)
        lam[core.unsqueeze(1), virt.unsqueeze(0)] = -delta[core.unsqueeze(1), virt.unsqueeze(0)]
        lam[virt.unsqueeze(1), core.unsqueeze(0)] = -delta[virt.unsqueeze(1), core.unsqueeze(0)]
        lam = back.T @ lam @ back
        return Fa + lam, Fb - lam

    if C0 is None:
        _, C = diag(H)
        C0 = (C, C)
    Da = C0[0][:, :na] @ C0[0][:, :na].T
    Db = C0[1][:, :nb] @ C0[1][:, :nb].T
    dia, dib = _SpinDIIS(), _SpinDIIS()
    E_old = Da_old = Db_old = None
    converged = False
    it = 0
    for it in range(1, max_iter + 1):
        Fa, Fb = engine.fock_u(Da, Db)
        if cuhf:
            Fa, Fb = constrain(Da, Db, Fa, Fb)
        Ra = Xt @ (S @ Da @ Fa - Fa @ Da @ S) @ X
        Rb = Xt @ (S @ Db @ Fb - Fb @ Db @ S) @ X
        vals = [0.5 * (torch.sum((Da + Db) * H) + torch.sum(Da * Fa) + torch.sum(Db * Fb)).reshape(1)]
        if Da_old is not None:
            vals.append(torch.sqrt(torch.mean((Da - Da_old) ** 2) + torch.mean((Db - Db_old) ** 2)).reshape(1))
        else:
            vals.append(torch.zeros(1, dtype=torch.float64, device=dev))
        vals.append(torch.stack([Ra.max(), Rb.max()]))
        ra, rb = Ra.reshape(-1), Rb.reshape(-1)
        vals.append(torch.stack([torch.dot(ra, r.reshape(-1)) for r in dia.res] + [torch.dot(ra, ra)]))
        vals.append(torch.stack([torch.dot(rb, r.reshape(-1)) for r in dib.res] + [torch.dot(rb, rb)]))
        host = torch.cat(vals).cpu().numpy()
        E = float(host[0]) + e_nuc
        if E_old is not None and abs(E - E_old) < e_tol and float(host[1]) < d_tol:
            converged = True
            break
        E_old, Da_old, Db_old = E, Da, Db
        Fxa, Fxb = Fa, Fb
        if it > 1:
            k = len(dia.res) + 1
            Fxa, _ = dia.extrapolate(Ra, Fa, host[4:4 + k], host[2])
            Fxb, _ = dib.extrapolate(Rb, Fb, host[4 + k:], host[3])
        ea, Ca = diag(Fxa)
        eb, Cb = diag(Fxb)
        if mom:
            Ca, ea = mom_order(Ca, ea, C0[0], na, S)
            Cb, eb = mom_order(Cb, eb, C0[1], nb, S)
        Da = Ca[:, :na] @ Ca[:, :na].T
        Db = Cb[:, :nb] @ Cb[:, :nb].T
    ea, Ca = diag(Fa)
    eb, Cb = diag(Fb)
    if mom:
        Ca, ea = _sort_occupied(*mom_order(Ca, ea, C0[0], na, S), na)
        Cb, eb = _sort_occupied(*mom_order(Cb, eb, C0[1], nb, S), nb)
    return SCFResult(E=E, Ca=Ca, Cb=Cb, ea=ea, eb=eb, Da=Da, Db=Db, Fa=Fa, Fb=Fb, iterations=it,
                     converged=converged)


def ump2(engine, res, eri=None, gemm="tc", nslice=6, scale=None):
    """Unrestricted MP2 correlation energy (Methods/mp2.py:43-101): same-spin
    0.25 sum ((ia|jb) - (ib|ja))^2 / D per spin and opposite-spin sum (ia|jb)^2 / D,
    with the orbital energies of the final Fock matrices; the integrals from the four
    quarter transforms of mp2_transform.  scale = (c_ss, c_os) weights the same-spin
    and opposite-spin parts (MP2_SCALES)."""
    mol = engine.mol
    na, nb = mol.NAlphaElectrons, mol.NBetaElectrons
    if eri is None:
        eri = engine.dense_eri() if gemm == "fp64" else engine.dense_eri_pairs(compact=True)
    Ca, Cb, ea, eb = res.Ca, res.Cb, res.ea, res.eb

    def same(C, e, o):
        if o == 0 or o == C.shape[1]:
            return 0.0
        g = mp2_transform(eri, C[:, :o].contiguous(), C[:, o:].contiguous(), gemm=gemm, nslice=nslice)
        s1, s2 = mp2_pair_sums(g, e[:o].contiguous(), e[o:].contiguous())
        return 0.5 * (s1 - s2)           # 0.25 sum ((ia|jb) - (ib|ja))^2 / D

    e_ab = 0.0
    if na and nb:
        g = mp2_transform(eri, Ca[:, :na].contiguous(), Ca[:, na:].contiguous(), gemm=gemm, nslice=nslice,
                          Co2=Cb[:, :nb].contiguous(), Cv2=Cb[:, nb:].contiguous())
        den = (ea[:na, None, None, None] - ea[None, na:, None, None] + eb[None, None, :nb, None]
               - eb[None, None, None, nb:])
        e_ab = float(torch.sum(g * g / den))
    if scale is not None:
        return scale[0] * (same(Ca, ea, na) + same(Cb, eb, nb)) + scale[1] * e_ab
    return same(Ca, ea, na) + same(Cb, eb, nb) + e_ab
