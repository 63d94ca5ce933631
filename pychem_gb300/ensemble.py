"""Batched RHF of an ensemble of small molecules in one set of launches.

Every molecule of the ensemble is a separate RHF problem (the upstream code runs them
one input section at a time, ``pychem.py:146-160``).  Here all of them share each
launch: shells of all molecules are concatenated, shell pairs and quartets are built
only inside a molecule, one-electron integrals see only the molecule's own nuclei, and
every matrix is a padded ``nbf_max x nbf_max`` block per molecule (padding AOs get
S = 1 and H = 1e3 on the diagonal, so they only form far-virtual orbitals).  The SCF
then runs on (batch, nbf_max, nbf_max) tensors: batched Fock digestion, batched FP64
Jacobi eigensolver (one CTA per molecule), batched DIIS.
"""
import ctypes
import time

import numpy as np
import torch

from . import _lib, eigen
from ._lib import BasisT
from .engine import GpuEngine, _ptr, _stream, pair_class
from .scf import SCFResult, diis_coefficients_batched

PAD_DIAG = 1.0e3


class EnsembleEngine(GpuEngine):
    def __init__(self, molecules, device="cuda", precision="fp64", fp32_below=1e-4, threshold=1e-8):
        self.mols = list(molecules)
        self.B = len(self.mols)
        self.nmax = max(m.NOrbitals for m in self.mols)
        self.mol = self.mols[0]
        super().__init__(self.mols[0], device=device, precision=precision, fp32_below=fp32_below,
                         threshold=threshold)

    # ---------------------------------------------------------------------------------
    def _upload_basis(self):
        arrs = [m.arrays() for m in self.mols]
        nsh = [len(a["sh_l"]) for a in arrs]
        npr = [len(a["pr_exp"]) for a in arrs]
        nat = [len(a["at_z"]) for a in arrs]
        sh_off = np.concatenate([[0], np.cumsum(nsh)[:-1]])
        pr_off = np.concatenate([[0], np.cumsum(npr)[:-1]])
        at_off = np.concatenate([[0], np.cumsum(nat)[:-1]])
        n2 = self.nmax * self.nmax
        a = dict(
            sh_l=np.concatenate([x["sh_l"] for x in arrs]).astype(np.int32),
            sh_nprim=np.concatenate([x["sh_nprim"] for x in arrs]).astype(np.int32),
            sh_prim=np.concatenate([x["sh_prim"] + o for x, o in zip(arrs, pr_off)]).astype(np.int32),
            sh_ao=np.concatenate([x["sh_ao"] for x in arrs]).astype(np.int32),
            sh_atom=np.concatenate([x["sh_atom"] + o for x, o in zip(arrs, at_off)]).astype(np.int32),
            sh_xyz=np.concatenate([x["sh_xyz"] for x in arrs]),
            pr_exp=np.concatenate([x["pr_exp"] for x in arrs]),
            pr_cc=np.concatenate([x["pr_cc"] for x in arrs]),
            at_xyz=np.concatenate([x["at_xyz"] for x in arrs]),
            at_z=np.concatenate([x["at_z"] for x in arrs]),
            sh_blk=np.concatenate([np.full(k, m * n2, dtype=np.int64) for m, k in enumerate(nsh)]),
            sh_at0=np.concatenate([np.full(k, o, dtype=np.int32) for k, o in zip(nsh, at_off)]),
            sh_nat=np.concatenate([np.full(k, na, dtype=np.int32) for k, na in zip(nsh, nat)]),
            sh_mol=np.concatenate([np.full(k, m, dtype=np.int32) for m, k in enumerate(nsh)]),
        )
        self.sh_off = sh_off
        self.h_basis = a
        self.d = {k: self._t(v) for k, v in a.items()}
        b = BasisT()
        b.nshell = len(a["sh_l"]); b.nprim = len(a["pr_exp"]); b.natom = len(a["at_z"]); b.nbf = self.nmax
        for k in ("sh_l", "sh_nprim", "sh_prim", "sh_ao", "sh_atom", "sh_xyz", "pr_exp", "pr_cc", "at_xyz", "at_z",
                  "sh_blk", "sh_at0", "sh_nat"):
            setattr(b, k, self.d[k].data_ptr())
        b.ld = self.nmax
        self.basis_t = b
        self.nbf = self.nmax

    def atom_table(self):
        if getattr(self, "_atoms", None) is None:
            self._atoms = atom_table(self.mols)
        return self._atoms

    def restrict(self, active):
        """Cut the quartet lists and integral stores down to the molecules with
        active[m] (host bool array); unrestrict() brings back the full ones."""
        if getattr(self, "_full", None) is None:
            self._full = (self.classes, self.stores)
        if getattr(self, "_pair_mol_dev", None) is None:
            self._pair_mol_dev = torch.as_tensor(self.pair_mol, dtype=torch.int64, device=self.dev)
        on = torch.as_tensor(active, device=self.dev)
        classes, stores = {}, {}
        for cls, rec in self.classes.items():
            nout = _lib.load().pcg_eri_class_nout(cls)
            new = {}
            for part, (tasks, nt) in rec.items():
                tv = tasks.view(nt, 2)
                keep = on[self._pair_mol_dev[tv[:, 0].long()]].nonzero().squeeze(1)
                if keep.numel() == 0:
                    continue
                new[part] = (tv.index_select(0, keep).reshape(-1), keep.numel())
                stores[(cls, part)] = self.stores[(cls, part)].view(nout, nt).index_select(1, keep).reshape(-1)
            if new:
                classes[cls] = new
        self.classes, self.stores = classes, stores

    def unrestrict(self):
        if getattr(self, "_full", None) is not None:
            self.classes, self.stores = self._full
            self._full = None

    def _pair_index(self):
        """Shell pairs a <= b inside each molecule (global shell indices)."""
        ia_all, ib_all = [], []
        for m, mol in enumerate(self.mols):
            n = mol.NCgtf
            ia, ib = np.triu_indices(n)
            ia_all.append(ia + self.sh_off[m])
            ib_all.append(ib + self.sh_off[m])
        return np.concatenate(ia_all), np.concatenate(ib_all)

    def _build_pairs(self):
        a = self.h_basis
        ia, ib = self._pair_index()
        la, lb = a["sh_l"][ia], a["sh_l"][ib]
        swap = lb > la
        A = np.where(swap, ib, ia).astype(np.int32)
        B = np.where(swap, ia, ib).astype(np.int32)
        self._finish_pairs(A, B)
        self.pair_mol = a["sh_mol"][A]

    # ---------------------------------------------------------------------------------
    def one_electron(self):
        n = self.nmax
        S = torch.zeros(self.B, n, n, dtype=torch.float64, device=self.dev)
        H = torch.zeros(self.B, n, n, dtype=torch.float64, device=self.dev)
        _lib.call("pcg_one_electron", ctypes.byref(self.basis_t), self.npair, _ptr(self.pd["A"]), _ptr(self.pd["B"]),
                  _ptr(S), _ptr(H), _stream())
        nb = torch.tensor([m.NOrbitals for m in self.mols], device=self.dev)
        pad = torch.arange(n, device=self.dev).unsqueeze(0) >= nb.unsqueeze(1)           # (B, n)
        S += torch.diag_embed(pad.to(torch.float64))
        H += torch.diag_embed(pad.to(torch.float64) * PAD_DIAG)
        self.S, self.H = S, H
        return S, H

    def _pair_molecule(self):
        if getattr(self, "_pair_mol_dev", None) is None:
            self._pair_mol_dev = torch.as_tensor(self.pair_mol, dtype=torch.int64, device=self.dev)
        return self._pair_mol_dev, self.B

    # ---------------------------------------------------------------------------------
    def fock(self, D, out=None, G=None):
        """Batched closed-shell Fock matrices (B, nmax, nmax)."""
        n = self.nmax
        if G is None:
            G = torch.zeros(self.B, n, n, dtype=torch.float64, device=self.dev)
        else:
            G.zero_()
        D = D.contiguous()
        for cls, rec in self.classes.items():
            for part, (tasks, ntask) in rec.items():
                _lib.call("pcg_digest_class", cls, ctypes.byref(self.basis_t), ctypes.byref(self.pairs_t), _ptr(tasks),
                          ntask, _ptr(self.stores[(cls, part)]), _ptr(D), _ptr(G), _stream())
        F = out if out is not None else torch.empty(self.B, n, n, dtype=torch.float64, device=self.dev)
        _lib.call("pcg_fock_build_batched", self.B, n, _ptr(self.H), _ptr(G), _ptr(F), _stream())
        return F

    def dense_eri(self):
        raise NotImplementedError("dense ERI tensors are built per molecule (GpuEngine)")


def atom_table(mols):
    """Per-atom rows of an ensemble, molecule by molecule: molecule index, first AO
    inside the molecule, AO count, Z, symbol, position (bohr); plus per molecule the
    index of its first atom and its atom count."""
    nat = np.array([m.NAtom for m in mols], dtype=np.int64)
    mol = np.repeat(np.arange(len(mols)), nat)
    sym = [a[0] for m in mols for a in m.atoms]
    z = np.array([a[1] for m in mols for a in m.atoms])
    xyz = np.array([a[2] for m in mols for a in m.atoms], dtype=np.float64).reshape(-1, 3)
    nao = np.array([k for m in mols for k in m.atom_nao()], dtype=np.int64)
    atom0 = np.concatenate([[0], np.cumsum(nat)[:-1]]).astype(np.int64)
    ao_glob = np.cumsum(nao) - nao
    ao0 = ao_glob - ao_glob[atom0][mol]
    return dict(mol=mol, ao0=ao0, nao=nao, z=z, sym=sym, xyz=xyz, atom0=atom0, nat=nat)


def sad_batch(eng):
    """Superposition of free-atom densities for every molecule, (B, nmax, nmax): one
    scatter per (element, basis) of the ensemble."""
    from .guess import atomic_density
    n = eng.nmax
    D = torch.zeros(eng.B, n, n, dtype=torch.float64, device=eng.dev)
    at = eng.atom_table()
    bas = np.array([m.Basis for m in eng.mols])[at["mol"]]
    groups = {}
    for k, key in enumerate(zip(at["sym"], bas)):
        groups.setdefault(key, []).append(k)
    for (s, b), rows in groups.items():
        rows = np.array(rows)
        Da = atomic_density(s, at["z"][rows[0]], b, eng.dev)
        k = Da.shape[0]
        r = torch.arange(k, device=eng.dev)
        m = torch.as_tensor(at["mol"][rows], device=eng.dev)[:, None, None]
        a = torch.as_tensor(at["ao0"][rows], device=eng.dev)[:, None, None]
        D[m, a + r[:, None], a + r[None, :]] = Da.unsqueeze(0).expand(len(rows), k, k)
    return D


def _dense_residual(F, Xa, Xta, Dp, dt):
    """Fock matrix in the orthonormal basis F' = X^T F X and the DIIS residual
    R = D'F' - F'D' (= X^T (S D F - F D S) X with D = X D' X^T), in dtype dt."""
    Fp = Xta.to(dt) @ F.to(dt) @ Xa.to(dt)
    P = Dp.to(dt) @ Fp
    return (P - P.transpose(-1, -2)).to(torch.float64)


def _dense_density(Fx, Xa, Xta, occa, Q, no, dt):
    """Eigenvectors Q' of X^T Fx X (dtype dt, starting from the previous Q), the AO
    density D = C_occ C_occ^T (C = X Q') and the orthonormal-basis density D'."""
    A = Xta.to(dt) @ Fx.to(dt) @ Xa.to(dt)
    if dt == torch.float32:
        _, V = eigen.eigh32(A, X_prev=Q.to(dt) if Q is not None else None)
    else:
        _, V = eigen.eigh(A, X_prev=Q)
    Vo = V[..., :no]
    mask = occa[:, :no].to(dt).unsqueeze(-2)
    Co = Xa.to(dt) @ Vo
    D = (Co * mask) @ Co.transpose(-1, -2)
    Dp = (Vo * mask) @ Vo.transpose(-1, -2)
    return V.to(torch.float64), D.to(torch.float64), Dp.to(torch.float64)


def rhf_batched(eng, max_iter=64, e_tol=1e-10, d_tol=1e-8, diis_size=8, guess="sad", D0=None, compact=0.5,
                dense_fp32_until=0.0, trace=None):
    """RHF of every molecule of a prepared EnsembleEngine.  Returns SCFResult with
    per-molecule arrays E, iterations (first iteration meeting the criteria), and C,
    eps, D (batch, nbf_max, ...).

    Molecules leave the iteration when they converge: the dense per-molecule work
    (residuals, DIIS, eigensolver) runs on the still-active rows only, and once the
    active molecules are at most `compact` of those the quartet lists cover, the lists
    and integral stores are cut down to the active molecules (the engine's full lists
    are restored on return).

    dense_fp32_until > 0 (mixed precision): while a molecule's DIIS residual has RMS
    above this value (1e-4 is the tested setting) and for at most 8 iterations, its
    dense steps (X^T F X, residual, eigensolver, density) run in FP32; after that, and
    for every iteration that can declare convergence, in FP64.
    Fock builds, DIIS extrapolation and energies are FP64 throughout, so the converged
    state is the FP64 one.

    trace: optional list that receives per iteration (iteration, active molecules, of
    them in FP32, seconds)."""
    B, n, dev = eng.B, eng.nmax, eng.dev
    S, H = eng.S, eng.H
    e_nuc = np.array([m.nuclear_repulsion() for m in eng.mols])
    nocc = torch.tensor([m.NAlphaElectrons for m in eng.mols], device=dev)
    for m in eng.mols:
        if m.NAlphaElectrons != m.NBetaElectrons:
            raise ValueError("rhf_batched needs closed-shell molecules")
    no = int(nocc.max())
    s, U = eigen.eigh(S)
    if float(s.min()) <= 1e-6:
        raise ValueError("linear dependence in an ensemble member; use GpuEngine for it")
    X = U * s.rsqrt().unsqueeze(-2)
    Xt = X.transpose(-1, -2).contiguous()
    occ = (torch.arange(n, device=dev).unsqueeze(0) < nocc.unsqueeze(1)).to(torch.float64)   # (B, n)

    Q = None
    if D0 is not None:
        D = D0.clone()
    elif guess == "sad":
        D = sad_batch(eng)
    else:
        Q, D, _ = _dense_density(H, X, Xt, occ, None, no, torch.float64)
        Q = None
    Dp = Xt @ S @ D @ S @ X
    # active rows: molecule ids `act` and their slices of every per-molecule tensor
    act = np.arange(B)
    Xa, Xta, Ha, occa, enuc_a = X, Xt, H, occ, e_nuc
    p32 = np.full(B, dense_fp32_until > 0)
    n32 = np.zeros(B, dtype=np.int64)
    Dfull = torch.zeros_like(S)
    Ffull = torch.empty_like(S)
    Gfull = torch.empty_like(S)
    F_fin = torch.empty_like(S)
    D_fin = torch.empty_like(S)
    focks, resids = [], []
    Bm = np.zeros((B, 0, 0))
    E_old = D_old = None
    done_at = np.zeros(B, dtype=np.int64)
    E_at = np.zeros(B)
    covered = B
    it = 0
    t_last = time.perf_counter()

    def groups(mask):
        out = []
        for flag, dt in ((True, torch.float32), (False, torch.float64)):
            rows = np.nonzero(mask == flag)[0]
            if len(rows):
                out.append((None if len(rows) == len(mask) else torch.as_tensor(rows, device=dev), dt))
        return out

    def take(t, rows):
        return t if rows is None else t.index_select(0, rows)

    try:
        for it in range(1, max_iter + 1):
            act_t = torch.as_tensor(act, device=dev)
            Dfull.index_copy_(0, act_t, D)
            eng.fock(Dfull, out=Ffull, G=Gfull)
            F = Ffull.index_select(0, act_t)
            R = torch.empty_like(F)
            for rows, dt in groups(p32):
                r_ = _dense_residual(take(F, rows), take(Xa, rows), take(Xta, rows), take(Dp, rows), dt)
                R = r_ if rows is None else R.index_copy_(0, rows, r_)
            Rf = R.reshape(len(act), -1)
            vals = [torch.sum(D * (Ha + F), dim=(1, 2))]
            vals.append(torch.sqrt(torch.mean((D - D_old) ** 2, dim=(1, 2))) if D_old is not None
                        else torch.zeros(len(act), dtype=torch.float64, device=dev))
            vals += [torch.sum(Rf * r.reshape(len(act), -1), dim=1) for r in resids] + [torch.sum(Rf * Rf, dim=1)]
            host = torch.stack(vals, dim=1).cpu().numpy()
            if trace is not None:
                now = time.perf_counter()
                trace.append((it, len(act), int(p32.sum()), now - t_last))
                t_last = now
            E = host[:, 0] + enuc_a
            if E_old is not None:
                conv = (np.abs(E - E_old) < e_tol) & (host[:, 1] < d_tol) & ~p32
                if conv.any():
                    ids = act[conv]
                    ct = torch.as_tensor(np.nonzero(conv)[0], device=dev)
                    it_ids = torch.as_tensor(ids, device=dev)
                    done_at[ids] = it
                    E_at[ids] = E[conv]
                    F_fin.index_copy_(0, it_ids, F.index_select(0, ct))
                    D_fin.index_copy_(0, it_ids, D.index_select(0, ct))
                    if conv.all():
                        act = act[:0]
                        break
                    keep = ~conv
                    kt = torch.as_tensor(np.nonzero(keep)[0], device=dev)
                    act = act[keep]
                    D, Dp, F, R = D[kt], Dp[kt], F[kt], R[kt]
                    Xa, Xta, Ha, occa = Xa[kt], Xta[kt], Ha[kt], occa[kt]
                    enuc_a, E, host, p32, n32 = enuc_a[keep], E[keep], host[keep], p32[keep], n32[keep]
                    Q = Q[kt] if Q is not None else None
                    focks = [f[kt] for f in focks]
                    resids = [r[kt] for r in resids]
                    Bm = Bm[keep]
                    if len(act) <= compact * covered:
                        mask = np.zeros(B, dtype=bool)
                        mask[act] = True
                        eng.restrict(mask)
                        covered = len(act)
            E_old, D_old = E, D
            # FP32 dense steps end once the residual is small, or after 8 iterations:
            # long FP32 phases (residual thresholds of 1e-5 and below) were seen to
            # steer single molecules into a higher SCF solution
            rms = np.sqrt(np.maximum(host[:, -1], 0.0) / (n * n))
            n32 += p32
            p32_new = p32 & (rms > dense_fp32_until) & (n32 < 8)
            switched = np.nonzero(p32 & ~p32_new)[0]
            p32 = p32_new
            if len(switched) and Q is not None:
                # the first FP64 step of a molecule starts from the identity (a full
                # Jacobi solve) instead of its FP32 eigenvectors, whose orthogonality
                # error would otherwise persist through X_prev
                sw = torch.as_tensor(switched, device=dev)
                Q.index_copy_(0, sw, torch.eye(n, dtype=torch.float64, device=dev).expand(len(switched), n, n))
            row = host[:, 2:]
            m = row.shape[1]
            Bn = np.zeros((len(act), m, m))
            Bn[:, :m - 1, :m - 1] = Bm
            Bn[:, m - 1, :] = row
            Bn[:, :, m - 1] = row
            focks.append(F)
            resids.append(R)
            Bm = Bn
            if len(focks) > diis_size:
                focks.pop(0); resids.pop(0)
                Bm = Bm[:, 1:, 1:]
            Fx = F
            k = len(focks)
            if k > 1:
                cw = torch.tensor(diis_coefficients_batched(Bm), dtype=torch.float64, device=dev)
                Fx = torch.einsum("bk,kbij->bij", cw, torch.stack(focks))
            Qn, Dn, Dpn = torch.empty_like(F), torch.empty_like(F), torch.empty_like(F)
            for rows, dt in groups(p32):
                out = _dense_density(take(Fx, rows), take(Xa, rows), take(Xta, rows), take(occa, rows),
                                     take(Q, rows) if Q is not None else None, no, dt)
                if rows is None:
                    Qn, Dn, Dpn = out
                else:
                    for dst, src in zip((Qn, Dn, Dpn), out):
                        dst.index_copy_(0, rows, src)
            Q, D, Dp = Qn, Dn, Dpn
    finally:
        eng.unrestrict()
    if len(act):
        at = torch.as_tensor(act, device=dev)
        E_at[act] = E
        F_fin.index_copy_(0, at, F)
        D_fin.index_copy_(0, at, D)
    still = done_at == 0
    eps, Qf = eigen.eigh(Xt @ F_fin @ X)
    return SCFResult(E=E_at, iterations=np.where(done_at > 0, done_at, it), converged=~still, C=X @ Qf, eps=eps,
                     D=D_fin, scf_iterations=it)
