"""CPU oracle for the RHF + MP2 path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg may
import this module, always as the checker.  It restates the upstream algorithm:

* AO bookkeeping: atoms in input order, shells in basis-library order, spherical
  functions in the rows of ``Data/transform_basis.py:3-12`` (``Util/structures.py:464-523``).
* one-electron S and H = T + V via ``hgp_oracle.c`` (``Methods/integrals.py:220-370``),
  assembled like ``Methods/hartree_fock.py:207-224``.
* canonical orthogonalisation X = U s^{-1/2}, eigenvalues sorted descending and
  s <= 1e-6 dropped (``Methods/hartree_fock.py:226-237``, ``Data/constants.py:34``).
* Schwarz-screened ERIs: diagonal (ab|ab) always, other unique shell quartets when
  max_ab * max_cd > 1e-8 (``Methods/hartree_fock.py:244-297``, ``Data/constants.py:31``).
* RHF through the UHF machinery with identical spins: J = einsum('cd,abcd->ab'),
  K = einsum('cb,abcd->ad') (``Methods/hartree_fock.py:329-355``), DIIS C1 on the
  residual X^T(SDF - FDS)X (``Methods/hf_extensions/diis.py:14-139``), energy
  0.5 sum(D_tot H + D_a F_a + D_b F_b) (``Methods/hartree_fock.py:188-201``).
  ``mode='reference'`` keeps upstream's choices (energy from the extrapolated Fock,
  |dE| stop only); ``mode='consistent'`` (the default checker) takes the energy from the
  Fock built from the current density and stops on |dE| < 1e-10 and D-RMS < 1e-8.
* MP2: closed-shell form of ``Methods/mp2.py:43-94`` (identical value for RHF).
* Open shells: UHF and CUHF along ``Methods/hartree_fock.py:23-142`` with the per-spin
  DIIS of ``Methods/hf_extensions/diis.py`` and the CUHF constraint of
  ``hartree_fock.py:359-391`` (natural orbitals of S^1/2 (D_tot/2) S^1/2), and UMP2 as
  ``Methods/mp2.py:43-101``; pinned by ``tests/test_oracle_open_shell.py``.
* NOCI: the CI matrix of ``Methods/noci.py:51-318`` (Lowdin pairing by numpy's SVD and
  the plain-dot-product phase rule as upstream, the no-, one- and two-zero element
  forms, the generalised eigenproblem) and the spin-flip orbital assembly of
  ``noci.py:127-146``; pinned by ``tests/test_noci_host.py``.
* Electron scattering: j0(S r12) integrals through ``hgp_oracle.c`` with the
  fundamentals of ``Methods/c_ints/two_electron_scattering.c`` and the Bessel scheme of
  ``spherical_bessel_j.c``, and the intensity contraction of
  ``Methods/properties.py:41-73``; pinned by ``tests/test_scattering_host.py``.
"""
import ctypes
import json
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
LIB_PATH = os.path.join(HERE, "libhgp_oracle.so")
BASIS_JSON = os.path.join(REPO, "pychem_gb300", "data", "basis_sets.json")
TO_BOHR = 1.8897161646320724        # Data/constants.py:2
INTEGRAL_THRESHOLD = 1.0e-8         # Data/constants.py:31
LINEAR_DEPENDENCE = 1.0e-6          # Data/constants.py:34
NELEC = {"H": 1, "HE": 2, "LI": 3, "BE": 4, "B": 5, "C": 6, "N": 7, "O": 8, "F": 9, "NE": 10}


class OrShell(ctypes.Structure):
    _fields_ = [("l", ctypes.c_int), ("nprim", ctypes.c_int), ("center", ctypes.c_double * 3),
                ("exps", ctypes.c_double * 16), ("ccs", ctypes.c_double * 16)]


def build(force=False):
    """Compile the C oracle (gcc, no GPU)."""
    src = os.path.join(HERE, "hgp_oracle.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.check_call(["gcc", "-O2", "-shared", "-fPIC", "-pthread", "-o", LIB_PATH, src, "-lm"])
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.POINTER
        L.oracle_eri_quartet.argtypes = [P(OrShell)] * 4 + [P(ctypes.c_double)]
        L.oracle_one_electron.argtypes = [P(OrShell), P(OrShell), ctypes.c_int, P(ctypes.c_double),
                                          P(ctypes.c_double)] + [P(ctypes.c_double)] * 3
        L.oracle_eri_list.argtypes = [P(OrShell), ctypes.c_int, P(ctypes.c_int)]
        L.oracle_eri_list.restype = ctypes.c_double
        L.oracle_boys.argtypes = [ctypes.c_int, ctypes.c_double, P(ctypes.c_double)]
        L.oracle_set_operator.argtypes = [ctypes.c_int, ctypes.c_double]
        L.oracle_sph_bessel.argtypes = [ctypes.c_int, ctypes.c_double, P(ctypes.c_double)]
        vp = ctypes.c_void_p
        L.oracle_eri_blocks.argtypes = [P(OrShell), ctypes.c_int, vp, vp, vp, ctypes.c_int]
        L.oracle_jk_packed.argtypes = [P(OrShell), vp, ctypes.c_int, vp, vp, vp, ctypes.c_int, vp, vp, vp, vp,
                                       ctypes.c_int]
        L.oracle_mp2_first_quarter.argtypes = [P(OrShell), vp, ctypes.c_int, vp, vp, vp, ctypes.c_int, ctypes.c_int,
                                               vp, vp, ctypes.c_int]
        assert L.oracle_sizeof_shell() == ctypes.sizeof(OrShell)
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def boys(mmax, T):
    out = np.zeros(mmax + 1)
    lib().oracle_boys(mmax, float(T), _dp(out))
    return out


class Basis:
    """Shells of a molecule in upstream AO order."""

    def __init__(self, atoms, basis_name, max_l=None):
        """atoms: list of (symbol, Z, x, y, z) with coordinates in bohr; max_l drops the
        shells above that angular momentum (Util/structures.py:815-826)."""
        with open(BASIS_JSON) as fh:
            lib_sets = json.load(fh)
        key = basis_name.replace("*", "s").replace("-", "").replace("(", "").replace(")", "").replace(",", "").upper()
        data = lib_sets[key]
        self.atoms = [(a[0].upper(), float(a[1]), np.array(a[2:5], dtype=float)) for a in atoms]
        self.shells = []      # (l, exps, ccs, centre, atom index)
        for ia, (sym, Z, xyz) in enumerate(self.atoms):
            for fn in data[sym]:
                l = fn[0]
                if max_l is not None and l > max_l:
                    continue
                exps = np.array([p[0] for p in fn[1:]], dtype=float)
                ccs = np.array([p[1] for p in fn[1:]], dtype=float)
                self.shells.append((l, exps, ccs, xyz, ia))
        self.offsets = []
        n = 0
        for s in self.shells:
            self.offsets.append(n)
            n += 2 * s[0] + 1
        self.nbf = n
        self.c = (OrShell * len(self.shells))()
        for i, (l, exps, ccs, xyz, _) in enumerate(self.shells):
            self.c[i].l = l
            self.c[i].nprim = len(exps)
            for k in range(3):
                self.c[i].center[k] = xyz[k]
            for k in range(len(exps)):
                self.c[i].exps[k] = exps[k]
                self.c[i].ccs[k] = ccs[k]
        self.nuc_xyz = np.ascontiguousarray([a[2] for a in self.atoms], dtype=float).reshape(-1, 3)
        self.nuc_z = np.array([a[1] for a in self.atoms], dtype=float)

    @property
    def nshell(self):
        return len(self.shells)

    def nelectrons(self, charge=0):
        return sum(NELEC[a[0]] for a in self.atoms) - charge

    def nuclear_repulsion(self):
        e = 0.0
        for i in range(len(self.atoms)):
            for j in range(i):
                r = np.linalg.norm(self.atoms[i][2] - self.atoms[j][2])
                e += self.atoms[i][1] * self.atoms[j][1] / r
        return e

    def shell_block(self, a, b, c, d):
        na, nb, nc, nd = (2 * self.shells[s][0] + 1 for s in (a, b, c, d))
        out = np.zeros(na * nb * nc * nd)
        rc = lib().oracle_eri_quartet(ctypes.byref(self.c[a]), ctypes.byref(self.c[b]),
                                      ctypes.byref(self.c[c]), ctypes.byref(self.c[d]), _dp(out))
        if rc != 0:
            raise ValueError("oracle supports shells up to d")
        return out.reshape(na, nb, nc, nd)

    def one_electron(self):
        S = np.zeros((self.nbf, self.nbf))
        H = np.zeros((self.nbf, self.nbf))
        for a in range(self.nshell):
            for b in range(a, self.nshell):
                na, nb = 2 * self.shells[a][0] + 1, 2 * self.shells[b][0] + 1
                s = np.zeros(na * nb); t = np.zeros(na * nb); v = np.zeros(na * nb)
                lib().oracle_one_electron(ctypes.byref(self.c[a]), ctypes.byref(self.c[b]), len(self.atoms),
                                          _dp(self.nuc_xyz), _dp(self.nuc_z), _dp(s), _dp(t), _dp(v))
                oa, ob = self.offsets[a], self.offsets[b]
                S[oa:oa + na, ob:ob + nb] = s.reshape(na, nb)
                S[ob:ob + nb, oa:oa + na] = s.reshape(na, nb).T
                h = (t + v).reshape(na, nb)
                H[oa:oa + na, ob:ob + nb] = h
                H[ob:ob + nb, oa:oa + na] = h.T
        return S, H

    def schwarz(self):
        """Per shell pair: max over functions of sqrt((mn|mn)) (hartree_fock.py:244-254)."""
        Q = np.zeros((self.nshell, self.nshell))
        for a in range(self.nshell):
            for b in range(a, self.nshell):
                blk = self.shell_block(a, b, a, b)
                na, nb = blk.shape[:2]
                diag = np.array([[blk[m, n, m, n] for n in range(nb)] for m in range(na)])
                Q[a, b] = Q[b, a] = math.sqrt(max(0.0, diag.max()))
        return Q

    def quartets(self, Q=None):
        """Canonical unique shell quartets kept by the upstream screening rule."""
        if Q is None:
            Q = self.schwarz()
        pairs = [(a, b) for a in range(self.nshell) for b in range(a, self.nshell)]
        out = []
        for i, (a, b) in enumerate(pairs):
            for j in range(i + 1):
                c, d = pairs[j]
                if i == j or Q[a, b] * Q[c, d] > INTEGRAL_THRESHOLD:
                    out.append((a, b, c, d))
        return out

    def quartet_array(self, Q=None):
        """quartets() as an int32 array (nq, 4), listed in the same order without a
        Python loop over quartets (for molecules with millions of them)."""
        if Q is None:
            Q = self.schwarz()
        ia, ib = np.triu_indices(self.nshell)
        q = Q[ia, ib]
        rows = []
        for i in range(len(ia)):
            js = np.nonzero(q[: i + 1] * q[i] > INTEGRAL_THRESHOLD)[0]
            if len(js) == 0 or js[-1] != i:
                js = np.append(js, i)
            rows.append(np.stack([np.full(len(js), ia[i]), np.full(len(js), ib[i]), ia[js], ib[js]], axis=1))
        return np.ascontiguousarray(np.concatenate(rows).astype(np.int32))

    def eri_dense(self, scattering=None):
        """Dense ERI tensor over the screened quartets (hartree_fock.py:241-327); with
        scattering = S the operator is j0(S r12) (the integrals of
        Methods/properties.py:20-23), screened by its own Schwarz bounds."""
        if scattering is not None:
            lib().oracle_set_operator(1, float(scattering))
            try:
                return self.eri_dense()
            finally:
                lib().oracle_set_operator(0, 0.0)
        n = self.nbf
        eri = np.zeros((n, n, n, n))
        for (a, b, c, d) in self.quartets():
            blk = self.shell_block(a, b, c, d)
            oa, ob, oc, od = (self.offsets[s] for s in (a, b, c, d))
            sa, sb, sc, sd = blk.shape
            A, B, C, D = slice(oa, oa + sa), slice(ob, ob + sb), slice(oc, oc + sc), slice(od, od + sd)
            eri[A, B, C, D] = blk
            eri[B, A, C, D] = blk.transpose(1, 0, 2, 3)
            eri[A, B, D, C] = blk.transpose(0, 1, 3, 2)
            eri[B, A, D, C] = blk.transpose(1, 0, 3, 2)
            eri[C, D, A, B] = blk.transpose(2, 3, 0, 1)
            eri[D, C, A, B] = blk.transpose(3, 2, 0, 1)
            eri[C, D, B, A] = blk.transpose(2, 3, 1, 0)
            eri[D, C, B, A] = blk.transpose(3, 2, 1, 0)
        return eri


class PackedStore:
    """The screened unique shell quartets of a Basis and their blocks, computed by the
    C oracle on several threads, for molecules whose dense N^4 tensor does not fit in
    host memory.  jk() and mp2_first_quarter() contract it without expanding it."""

    def __init__(self, basis, nthreads=None, Q=None, quads=None):
        """quads: an explicit (nq, 4) quartet list instead of the screened one (a
        sample, for timing)."""
        self.basis = basis
        self.nthreads = nthreads or os.cpu_count() or 1
        self.quads = basis.quartet_array(Q) if quads is None else np.ascontiguousarray(quads, dtype=np.int32)
        ls = np.array([s[0] for s in basis.shells])
        dims = 2 * ls + 1
        size = dims[self.quads[:, 0]] * dims[self.quads[:, 1]] * dims[self.quads[:, 2]] * dims[self.quads[:, 3]]
        self.boff = np.ascontiguousarray(np.concatenate([[0], np.cumsum(size)[:-1]]).astype(np.int64))
        self.blocks = np.empty(int(size.sum()))
        self.ao = np.ascontiguousarray(basis.offsets, dtype=np.int32)
        self.n = basis.nbf
        rc = lib().oracle_eri_blocks(basis.c, len(self.quads), self.quads.ctypes.data, self.boff.ctypes.data,
                                     self.blocks.ctypes.data, self.nthreads)
        if rc != 0:
            raise RuntimeError("oracle_eri_blocks failed")

    @property
    def nquartets(self):
        return len(self.quads)

    def jk(self, Dj, Dk):
        """J = einsum('cd,abcd->ab', Dj, ERI), K = einsum('cb,abcd->ad', Dk, ERI)."""
        n = self.n
        Dj, Dk = np.ascontiguousarray(Dj, dtype=float), np.ascontiguousarray(Dk, dtype=float)
        J, K = np.empty((n, n)), np.empty((n, n))
        rc = lib().oracle_jk_packed(self.basis.c, self.ao.ctypes.data, len(self.quads), self.quads.ctypes.data,
                                    self.boff.ctypes.data, self.blocks.ctypes.data, n, Dj.ctypes.data,
                                    Dk.ctypes.data, J.ctypes.data, K.ctypes.data, self.nthreads)
        if rc != 0:
            raise RuntimeError("oracle_jk_packed failed")
        return J, K

    def mp2_first_quarter(self, Co):
        """T[i][nu][rs] = sum_mu Co[mu][i] (mu nu | r s), rs = r(r+1)/2 + s, r >= s."""
        n, o = Co.shape
        Co = np.ascontiguousarray(Co, dtype=float)
        T = np.zeros((o, n, n * (n + 1) // 2))
        rc = lib().oracle_mp2_first_quarter(self.basis.c, self.ao.ctypes.data, len(self.quads),
                                            self.quads.ctypes.data, self.boff.ctypes.data, self.blocks.ctypes.data,
                                            n, o, Co.ctypes.data, T.ctypes.data, self.nthreads)
        if rc != 0:
            raise RuntimeError("oracle_mp2_first_quarter failed")
        return T


def rmp2_packed(C, eps, store, nocc):
    """rmp2() over a PackedStore: first quarter transform from the store (C), the
    other three by dense products one occupied orbital at a time, so that neither the
    dense AO tensor nor a full N^3 o intermediate is held."""
    n = C.shape[0]
    Co, Cv = C[:, :nocc], C[:, nocc:]
    v = Cv.shape[1]
    T1 = store.mp2_first_quarter(Co)                     # (i, nu, rs)
    r, s_ = np.tril_indices(n)
    ovov = np.empty((nocc, v, nocc, v))
    M = np.zeros((v, n, n))
    for i in range(nocc):
        T2 = Cv.T @ T1[i]                                # (a, rs)
        M[:, r, s_] = T2
        M[:, s_, r] = T2
        ovov[i] = np.einsum("alk,lj,kb->ajb", M, Co, Cv, optimize=True)
    del T1
    eo, ev = eps[:nocc], eps[nocc:]
    denom = eo[:, None, None, None] - ev[None, :, None, None] + eo[None, None, :, None] - ev[None, None, None, :]
    return float(np.sum(ovov * (2.0 * ovov - ovov.transpose(0, 3, 2, 1)) / denom))


def pack8(eri):
    """8-fold unique packing (i>=j, k>=l, ij>=kl), pair index i(i+1)/2+j."""
    n = eri.shape[0]
    ii, jj = np.tril_indices(n)
    P, Q = np.tril_indices(len(ii))
    return eri[ii[P], jj[P], ii[Q], jj[Q]].copy()


def unpack8(packed, n):
    ii, jj = np.tril_indices(n)
    npair = len(ii)
    M = np.zeros((npair, npair))
    P, Q = np.tril_indices(npair)
    M[P, Q] = packed
    M[Q, P] = packed
    eri = np.zeros((n, n, n, n))
    eri[ii[:, None], jj[:, None], ii[None, :], jj[None, :]] = M
    eri[jj[:, None], ii[:, None], ii[None, :], jj[None, :]] = M
    eri[ii[:, None], jj[:, None], jj[None, :], ii[None, :]] = M
    eri[jj[:, None], ii[:, None], jj[None, :], ii[None, :]] = M
    return eri


def orthogonaliser(S):
    s, U = np.linalg.eigh(S)
    order = s.argsort()[::-1]
    U = U[:, order]
    s = s[order]
    keep = s > LINEAR_DEPENDENCE
    return U[:, keep] * (s[keep] ** -0.5)


def rhf(S, H, eri, nocc, e_nuc, mode="consistent", max_iter=200, e_tol=1e-10, d_tol=1e-8,
        diis_size=None, D0=None, store=None):
    """Returns dict(E, C, eps, D, iterations, converged).  With a PackedStore in
    ``store`` (and eri None) the Coulomb and exchange matrices come from it."""
    X = orthogonaliser(S)
    Xt = X.T

    def diag(F):
        e, Cp = np.linalg.eigh(Xt @ F @ X)
        return e, X @ Cp

    if D0 is None:
        eps, C = diag(H)
        D = C[:, :nocc] @ C[:, :nocc].T
    else:
        D = D0.copy()
    F = H.copy()

    def fock(D):
        if store is not None:
            J, K = store.jk(2.0 * D, D)
            return H + J - K
        J = np.einsum("cd,abcd->ab", 2.0 * D, eri, optimize=True)
        K = np.einsum("cb,abcd->ad", D, eri, optimize=True)
        return H + J - K

    def energy(D, F):
        return 0.5 * np.sum(2.0 * D * H) + np.sum(D * F) + e_nuc

    E = energy(D, F if mode == "reference" else fock(D))
    focks, resids = [], []
    converged = False
    it = 0
    for it in range(1, max_iter + 1):
        F = fock(D)
        E_cons = energy(D, F)
        R = Xt @ (S @ D @ F - F @ D @ S) @ X
        Fx = F
        if it > 1 and (mode == "consistent" or abs(R.max()) < 0.5):
            focks.append(F.copy())
            resids.append(R.copy())
            if diis_size and len(focks) > diis_size:
                focks.pop(0); resids.pop(0)
            if len(focks) > 1:
                while True:
                    m = len(focks)
                    B = -np.ones((m + 1, m + 1))
                    B[m, m] = 0.0
                    for i in range(m):
                        for j in range(m):
                            B[i, j] = np.sum(resids[i] * resids[j])
                    ev = np.abs(np.linalg.eigvals(B))
                    if ev.min() > 0 and ev.max() / ev.min() <= 1e7 or m <= 2:
                        break
                    focks.pop(0); resids.pop(0)
                rhs = np.zeros(m + 1)
                rhs[m] = -1.0
                c = np.linalg.solve(B, rhs)[:m]
                Fx = sum(ci * Fi for ci, Fi in zip(c, focks))
        eps, C = diag(Fx)
        D_new = C[:, :nocc] @ C[:, :nocc].T
        if mode == "reference":
            E_new = energy(D_new, Fx)
        else:
            E_new = energy(D_new, fock(D_new))
        dE = E_new - E
        drms = math.sqrt(np.mean((D_new - D) ** 2))
        D, E = D_new, E_new
        if mode == "reference":
            if abs(dE) < e_tol:
                converged = True
                break
        elif abs(dE) < e_tol and drms < d_tol:
            converged = True
            break
    F = fock(D)
    eps, C = diag(F)
    return dict(E=E, C=C, eps=eps, D=D, iterations=it, converged=converged, F=F)


def rmp2(C, eps, eri, nocc):
    """Closed-shell MP2 correlation energy from the dense AO ERI tensor."""
    Co, Cv = C[:, :nocc], C[:, nocc:]
    ovov = np.einsum("pi,qa,rj,sb,pqrs->iajb", Co, Cv, Co, Cv, eri, optimize=True)
    eo, ev = eps[:nocc], eps[nocc:]
    denom = eo[:, None, None, None] - ev[None, :, None, None] + eo[None, None, :, None] - ev[None, None, None, :]
    return float(np.sum(ovov * (2.0 * ovov - ovov.transpose(0, 3, 2, 1)) / denom))


def half_overlap(S):
    """S^{1/2} over the eigenvalues above the linear-dependence cut, as
    Methods/hartree_fock.py:226-237 stores it (molecule.S)."""
    s, U = np.linalg.eigh(S)
    keep = s > LINEAR_DEPENDENCE
    return (U[:, keep] * np.sqrt(s[keep])) @ U[:, keep].T


def cuhf_constraint(S, Da, Db, Fa, Fb, na, nb, spaces=None):
    """The CUHF constraint of Methods/hartree_fock.py:359-391 (constrain_UHF): natural
    orbitals from eigh(S^1/2 (D_tot / 2) S^1/2) with coefficients (S^1/2)^-1 V, and the
    core-virtual block of (F_a - F_b) / 2 in that basis cancelled: F_a + L, F_b - L.
    spaces = (core, active): the counts of doubly and singly occupied positions of the
    state's occupancy lists (hartree_fock.py:361-365); (nb, na - nb) for aufbau states."""
    Sh = half_overlap(S)
    P = Sh @ ((Da + Db) / 2.0) @ Sh
    vals, vecs = np.linalg.eigh(P)
    Cno = np.linalg.inv(Sh) @ vecs
    back = np.linalg.inv(Cno)
    idx = vals.argsort()[::-1]
    nc, nact = spaces if spaces is not None else (nb, na - nb)
    core, virt = idx[:nc], idx[nc + nact:]
    delta = Cno.T @ ((Fa - Fb) / 2.0) @ Cno
    lam = np.zeros_like(delta)
    lam[np.ix_(core, virt)] = -delta[np.ix_(core, virt)]
    lam[np.ix_(virt, core)] = -delta[np.ix_(virt, core)]
    lam = back.T @ lam @ back
    return Fa + lam, Fb - lam


class _SpinDIIS:
    """Methods/hf_extensions/diis.py:14-154 for one spin: a residual enters the space
    only while its largest element is below 0.5 (diis.py:22,32-34), C1 coefficients
    (diis.py:108-112), the oldest vectors dropped while the B matrix's eigenvalue
    condition number exceeds 1e7 (diis.py:87-96, Data/constants.py:36)."""

    def __init__(self):
        self.res, self.focks = [], []

    def extrapolate(self, R, F):
        if not abs(R.max()) < 0.5:
            return F
        self.res.append(R)
        self.focks.append(F)
        if len(self.res) < 2:
            return F
        while True:
            m = len(self.res)
            B = -np.ones((m + 1, m + 1))
            B[m, m] = 0.0
            for i in range(m):
                for j in range(m):
                    B[i, j] = np.trace(self.res[i] @ self.res[j].T)
            ev = np.abs(np.linalg.eigvals(B))
            cond = ev.max() / ev.min() if ev.min() > 0 else np.inf
            if cond <= 1e7 or m == 1:
                break
            self.res.pop(0); self.focks.pop(0)
        rhs = np.zeros(m + 1)
        rhs[m] = -1.0
        c = np.linalg.solve(B, rhs)[:m]
        return sum(ci * Fi for ci, Fi in zip(c, self.focks))


def mom_order(C_new, e_new, C_ref, n, S):
    """Methods/hf_extensions/mom.py:6-47: order the new orbitals by decreasing
    |sum_j <ref_j|new_i>| over the n occupied reference orbitals (stable sort)."""
    p = np.abs((C_ref[:, :n].T @ S @ C_new).sum(axis=0))
    order = np.argsort(-p, kind="stable")
    return C_new[:, order], e_new[order]


def uhf(S, H, eri, na, nb, e_nuc, cuhf=False, max_iter=300, e_tol=1e-11, d_tol=1e-9, C0=None, mom=False,
        cuhf_spaces=None):
    """Unrestricted (or constrained, cuhf=True) Hartree-Fock along the upstream path of
    Methods/hartree_fock.py:23-142: core-Hamiltonian guess for both spins,
    F_s = H + J[D_a + D_b] - K[D_s] (hartree_fock.py:329-355), the optional CUHF
    constraint (hartree_fock.py:359-391), DIIS per spin (_SpinDIIS), aufbau occupation,
    energy 0.5 sum(D_tot H + D_a F_a + D_b F_b) (hartree_fock.py:188-201) taken here
    from the Fock matrices of the current densities; stops on |dE| < e_tol and a
    density change below d_tol.  C0 = (Ca, Cb): starting orbitals (occupied columns
    first) instead of the core guess; mom: occupy by maximum overlap with C0's
    occupied orbitals (the FIXED reference of Methods/hf_extensions/mom.py) instead of
    aufbau; cuhf_spaces: the constraint's (core, active) counts (cuhf_constraint).
    Returns dict(E, Ca, Cb, ea, eb, Da, Db, Fa, Fb, iterations, converged)."""
    X = orthogonaliser(S)
    Xt = X.T

    def diag(F):
        e, Cp = np.linalg.eigh(Xt @ F @ X)
        return e, X @ Cp

    if C0 is None:
        _, C = diag(H)
        C0 = (C, C)
    Da = C0[0][:, :na] @ C0[0][:, :na].T
    Db = C0[1][:, :nb] @ C0[1][:, :nb].T

    def focks(Da, Db):
        J = np.einsum("cd,abcd->ab", Da + Db, eri, optimize=True)
        Ka = np.einsum("cb,abcd->ad", Da, eri, optimize=True)
        Kb = np.einsum("cb,abcd->ad", Db, eri, optimize=True)
        Fa, Fb = H + J - Ka, H + J - Kb
        if cuhf:
            Fa, Fb = cuhf_constraint(S, Da, Db, Fa, Fb, na, nb, cuhf_spaces)
        return Fa, Fb

    def energy(Da, Db, Fa, Fb):
        return 0.5 * (np.sum((Da + Db) * H) + np.sum(Da * Fa) + np.sum(Db * Fb)) + e_nuc

    da, db = _SpinDIIS(), _SpinDIIS()
    E_old = None
    drms = np.inf
    converged = False
    it = 0
    for it in range(1, max_iter + 1):
        Fa, Fb = focks(Da, Db)
        E = energy(Da, Db, Fa, Fb)
        if E_old is not None and abs(E - E_old) < e_tol and drms < d_tol:
            converged = True
            break
        E_old = E
        Fxa, Fxb = Fa, Fb
        if it > 1:
            Fxa = da.extrapolate(Xt @ (S @ Da @ Fa - Fa @ Da @ S) @ X, Fa)
            Fxb = db.extrapolate(Xt @ (S @ Db @ Fb - Fb @ Db @ S) @ X, Fb)
        ea, Ca = diag(Fxa)
        eb, Cb = diag(Fxb)
        if mom:
            Ca, ea = mom_order(Ca, ea, C0[0], na, S)
            Cb, eb = mom_order(Cb, eb, C0[1], nb, S)
        Da_new = Ca[:, :na] @ Ca[:, :na].T
        Db_new = Cb[:, :nb] @ Cb[:, :nb].T
        drms = math.sqrt(np.mean((Da_new - Da) ** 2) + np.mean((Db_new - Db) ** 2))
        Da, Db = Da_new, Db_new
    ea, Ca = diag(Fa)
    eb, Cb = diag(Fb)
    if mom:
        Ca, ea = mom_order(Ca, ea, C0[0], na, S)
        Cb, eb = mom_order(Cb, eb, C0[1], nb, S)
    return dict(E=E, Ca=Ca, Cb=Cb, ea=ea, eb=eb, Da=Da, Db=Db, Fa=Fa, Fb=Fb, iterations=it, converged=converged)


def ump2(Ca, Cb, ea, eb, eri, na, nb, scale=None):
    """Unrestricted MP2 correlation energy, Methods/mp2.py:43-101: same-spin
    sum over i >= j, p >= q of (<ip|jq> - <iq|jp>)^2 / D, opposite-spin sum of
    <ip|jq>^2 / D, with the orbital energies of the final Fock matrices; scale =
    (c_ss, c_os) weights the two parts (SCS / SOS, Methods/mp2.py:97-107)."""
    def mo(C1, C2, o1, o2):
        return np.einsum("pi,qa,rj,sb,pqrs->iajb", C1[:, :o1], C1[:, o1:], C2[:, :o2], C2[:, o2:], eri, optimize=True)

    def same(C, e, o):
        g = mo(C, C, o, o)
        eo, ev = e[:o], e[o:]
        den = eo[:, None, None, None] - ev[None, :, None, None] + eo[None, None, :, None] - ev[None, None, None, :]
        t = g - g.transpose(0, 3, 2, 1)
        return 0.25 * float(np.sum(t * t / den))

    g = mo(Ca, Cb, na, nb)
    den = (ea[:na, None, None, None] - ea[None, na:, None, None] + eb[None, None, :nb, None]
           - eb[None, None, None, nb:])
    e_ss, e_os = same(Ca, ea, na) + same(Cb, eb, nb), float(np.sum(g * g / den))
    if scale is not None:
        return scale[0] * e_ss + scale[1] * e_os
    return e_ss + e_os


# ------------------------------------------------------------------------------------
# NOCI (Methods/noci.py)
# ------------------------------------------------------------------------------------
NOCI_THRESH = 1.0e-8                # Data/constants.py:37


def noci_biorthogonalize(C1, C2, S, n):
    """Methods/noci.py:183-205: Lowdin-paired occupied orbitals from the SVD of
    C1_o^T S C2_o; a pair whose plain (unit-metric) dot product is negative has the
    second orbital's sign flipped."""
    A, B = C1[:, :n], C2[:, :n]
    U, _, Vt = np.linalg.svd(A.T @ S @ B)
    A2, B2 = A @ U, B @ Vt.T
    flip = np.einsum("pi,pi->i", A2, B2) < 0
    B2[:, flip] *= -1.0
    return A2, B2


def noci_coulomb_exchange(Wa, Wb, eri):
    """Methods/hartree_fock.py:345-347 on co-densities: J[W_a + W_b] and the exchange
    matrices -K[W_s] with K_ad = sum_bc (ab|cd) W_cb."""
    J = np.einsum("cd,abcd->ab", Wa + Wb, eri, optimize=True)
    Xa = np.einsum("cb,abcd->ad", -Wa, eri, optimize=True)
    Xb = np.einsum("cb,abcd->ad", -Wb, eri, optimize=True)
    return J, Xa, Xb


def noci_element(Ca1, Cb1, Ca2, Cb2, S, H, eri, na, nb, e_nuc):
    """One CI matrix element and overlap, Methods/noci.py:63-106: Lowdin pairing of
    each spin, then noci_element_paired."""
    a1, a2 = noci_biorthogonalize(Ca1, Ca2, S, na)
    b1, b2 = noci_biorthogonalize(Cb1, Cb2, S, nb)
    return noci_element_paired(a1, a2, b1, b2, S, H, eri, na, nb, e_nuc)


def noci_zero_counts(a1, a2, b1, b2, S):
    """Numbers of paired overlaps at or below NOCI_THRESH in each spin."""
    ov_a = np.diagonal(a1.T @ S @ a2)
    ov_b = np.diagonal(b1.T @ S @ b2)
    return int((ov_a <= NOCI_THRESH).sum()), int((ov_b <= NOCI_THRESH).sum())


def noci_element_paired(a1, a2, b1, b2, S, H, eri, na, nb, e_nuc):
    """The element from given paired orbitals, Methods/noci.py:65-106 with the helpers
    of noci.py:207-318: reduced overlap over the paired overlaps above NOCI_THRESH,
    the no-zero, one-zero and two-zero forms (the two-zero form uses the first zero's
    index in both spins, as upstream), 0 for more zeros; then times the reduced
    overlap plus E_nuc times the determinant overlap.  With two zeros in one spin the
    zero singular value is degenerate and the upstream form depends on the basis the
    SVD picks inside that null space; given the same pairing it is exact."""
    a1, a2, b1, b2 = a1.copy(), a2.copy(), b1.copy(), b2.copy()
    core_a = a1.T @ H @ a2
    core_b = b1.T @ H @ b2
    ov_a = np.diagonal(a1.T @ S @ a2).copy()
    ov_b = np.diagonal(b1.T @ S @ b2).copy()
    s_state = float(np.prod(ov_a) * np.prod(ov_b))
    reduced = 1.0
    zeros = []
    for spin, ov in (("a", ov_a), ("b", ov_b)):
        for i, o in enumerate(ov):
            if o > NOCI_THRESH:
                reduced *= o
            else:
                zeros.append((i, spin))
    if na > nb:                      # noci.py:81-84: beta padded to the alpha width
        ov_b = np.concatenate([ov_b, np.ones(na - nb)])
        b1 = np.concatenate([b1, np.zeros((b1.shape[0], na - nb))], axis=1)
        b2 = np.concatenate([b2, np.zeros((b2.shape[0], na - nb))], axis=1)

    def weighted(x1, x2, ov):
        keep = ov > NOCI_THRESH
        return (x1[:, keep] / ov[keep]) @ x2[:, keep].T

    def inner(m1, m2):
        return float(np.sum(m1 * m2))

    if len(zeros) == 0:
        Wa, Wb = weighted(a1, a2, ov_a), weighted(b1, b2, ov_b)
        J, Xa, Xb = noci_coulomb_exchange(Wa, Wb, eri)
        elem = 0.5 * (inner(Wa + Wb, J) + inner(Wa, Xa) + inner(Wb, Xb))
        elem += sum(core_a[i, i] / ov_a[i] for i in range(na) if ov_a[i] > NOCI_THRESH)
        elem += sum(core_b[i, i] / ov_b[i] for i in range(nb) if ov_b[i] > NOCI_THRESH)
    elif len(zeros) == 1:
        z, spin = zeros[0]
        Wa, Wb = weighted(a1, a2, ov_a), weighted(b1, b2, ov_b)
        J, Xa, Xb = noci_coulomb_exchange(Wa, Wb, eri)
        x1, x2, X, core = (a1, a2, Xa, core_a) if spin == "a" else (b1, b2, Xb, core_b)
        P = np.outer(x1[:, z], x2[:, z])
        elem = inner(P, J) + inner(P, X) + core[z, z]
    elif len(zeros) == 2:
        z, spin = zeros[0]
        Pa, Pb = np.outer(a1[:, z], a2[:, z]), np.outer(b1[:, z], b2[:, z])
        J, Xa, Xb = noci_coulomb_exchange(Pa, Pb, eri)
        P, X = (Pa, Xa) if spin == "a" else (Pb, Xb)
        elem = inner(P, J) + inner(P, X)
    else:
        elem = 0.0
    return elem * reduced + e_nuc * s_state, s_state


def noci(dets_a, dets_b, S, H, eri, na, nb, e_nuc):
    """Methods/noci.py:51-109: the CI matrix and overlap over the determinants (lower
    triangle computed with state i as the bra, mirrored), then the generalised
    symmetric eigenproblem (scipy.linalg.eigh).  Returns (energies, vectors, Hci, Sci)."""
    from scipy.linalg import eigh
    m = len(dets_a)
    Hci = np.zeros((m, m))
    Sci = np.zeros((m, m))
    for i in range(m):
        for j in range(i + 1):
            h, s = noci_element(dets_a[i], dets_b[i], dets_a[j], dets_b[j], S, H, eri, na, nb, e_nuc)
            Hci[i, j] = Hci[j, i] = h
            Sci[i, j] = Sci[j, i] = s
    e, v = eigh(Hci, Sci)
    return e, v, Hci, Sci


def noci_assemble(occupancy, C, hf_occupancy):
    """Methods/noci.py:127-146: orbitals of a spin-flip determinant from a Hartree-Fock
    state's orbitals: occupied columns (each must be occupied in that state) first in
    order, the unoccupied ones after them."""
    occupancy = list(occupancy)
    out = np.zeros_like(C)
    n_occ = sum(occupancy)
    k_occ, k_virt = 0, n_occ
    for i, o in enumerate(occupancy):
        if o == 0:
            out[:, k_virt] = C[:, i]
            k_virt += 1
        elif o == 1 and hf_occupancy[i] == 1:
            out[:, k_occ] = C[:, i]
            k_occ += 1
        else:
            raise ValueError("spin-flip determinant needs an orbital its Hartree-Fock state leaves empty")
    return out


# ------------------------------------------------------------------------------------
# Electron scattering (Methods/properties.py)
# ------------------------------------------------------------------------------------
def sph_bessel_scaled(lmax, z):
    """z^-m j_m(z), m = 0..lmax, by the piecewise scheme of spherical_bessel_j.c."""
    out = np.zeros(lmax + 1)
    lib().oracle_sph_bessel(lmax, float(z), _dp(out))
    return out


def scattering_intensity(Da, Db, eri_S, n_electrons):
    """Total scattering intensity of one state at one momentum transfer,
    Methods/properties.py:20-23,41-73: N + sum_abcd [P_ab P_cd - (Pa_ad Pa_cb +
    Pb_ad Pb_cb)] (ab|j0(S r12)|cd)."""
    P = Da + Db
    v = np.einsum("ab,cd,abcd->", P, P, eri_S, optimize=True)
    v -= np.einsum("ad,cb,abcd->", Da, Da, eri_S, optimize=True)
    v -= np.einsum("ad,cb,abcd->", Db, Db, eri_S, optimize=True)
    return n_electrons + float(v)
