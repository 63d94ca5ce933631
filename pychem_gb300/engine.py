"""Whole-molecule GPU integral engine: pair data, one-electron matrices, Schwarz pass,
screened shell-quartet task lists, in-core ERI store and closed-shell Fock digestion.

Replaces the per-shell-pair / per-quartet Python loops of the upstream
``Methods/hartree_fock.py:207-355`` (``make_core_matrices``, ``evaluate_2e_ints``,
``make_coulomb_exchange_matrices``) with batched launches of the C ABI in
``include/pychem_gb300.h``.  Device memory and streams come from PyTorch; all
arithmetic runs in the library's kernels.
"""
import ctypes
import math

import numpy as np
import torch

from . import _lib
from ._lib import BasisT, PairsT

INTEGRAL_THRESHOLD = 1.0e-8   # Data/constants.py:31
N_SPHER = [1, 3, 5]


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None and t.numel() else ctypes.c_void_p(0)


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def pair_class(la, lb):
    return la * (la + 1) // 2 + lb


def pair_colmap(n, pmap, device):
    """(n x n int32) where each AO pair (a, b) sits in a pair-packed row: pmap[pair(a, b)]
    (-1: not stored), or pair(a, b) itself when pmap is None (pcg_pair_colmap)."""
    cm = torch.empty(n * n, dtype=torch.int32, device=device)
    _lib.call("pcg_pair_colmap", n, _ptr(pmap), _ptr(cm), _stream())
    return cm


def plan_quartets(Q, kind, mol, nmol, class_table, thr, thr32, kind_work=None):
    """Screened canonical quartet plan (Methods/hartree_fock.py:241-312: the quartet
    loop, the Schwarz test Q_ab Q_cd > threshold, and the diagonal quartet that is
    always computed), with tensor operations on Q's device.

    Q, kind, mol: per shell pair its Schwarz factor, kind index (kinds ordered by
    (pair class, nA, nB)) and molecule; class_table[kb, kc] the ERI class of bra kind
    kb with ket kind kc <= kb.  Pairs are sorted by (kind, molecule, -Q); for a bra
    pair and a ket kind the kets of the bra's molecule are one segment of that order
    and the screened kets a prefix of it, whose length is found by bisection on the
    exact predicate.  Each quartet is listed once: bra kind >= ket kind, and within
    one kind the ket comes no later than the bra in the order, the bra's own diagonal
    quartet always included.  Quartets with Q_ab Q_cd <= thr32 (mixed precision, not
    the appended diagonal) form the FP32 part.

    Returns ([(class, part, bra pair, off, qstart, diag), ...], ket_list): rows of a
    class and part ordered by (bra kind, ket kind, bra position) -- buckets of uniform
    primitive counts -- with bra pair ids, task offsets off (int64, rows + 1, starting
    at 0), first ket position qstart in ket_list (the pair ids in sorted order) and
    the diagonal flag; row r covers tasks [off[r], off[r+1]).  With kind_work (work
    per pair of each kind, e.g. its primitive-pair count) the buckets run in
    decreasing work per quartet, so a launch's heaviest CTAs start first and the light
    ones fill its tail."""
    dev = Q.device
    nk = int(class_table.shape[0])
    o = torch.sort(-Q, stable=True).indices
    o = o[torch.sort(mol[o], stable=True).indices]
    o = o[torch.sort(kind[o], stable=True).indices]
    Qs, ks, ms = Q[o], kind[o], mol[o]
    seg_key = ks * nmol + ms
    npair = o.numel()
    # rows: (position of the bra in the order, ket kind <= bra kind)
    pos = torch.repeat_interleave(torch.arange(npair, device=dev), ks + 1)
    first = torch.cumsum(ks + 1, 0) - (ks + 1)
    kk = torch.arange(pos.numel(), device=dev) - first[pos]
    kb = ks[pos]
    key = (kb * nk + kk) * npair + pos
    if kind_work is not None:
        w = kind_work[kb] * kind_work[kk]
        key = (int(w.max()) - w) * (nk * nk * npair) + key
    ro = torch.sort(key).indices
    pos, kk, kb = pos[ro], kk[ro], kb[ro]
    qb = Qs[pos]
    key = kk * nmol + ms[pos]
    lo = torch.searchsorted(seg_key, key, right=False)
    hi = torch.searchsorted(seg_key, key, right=True)
    nbits = int((hi - lo).max()).bit_length() + 1 if pos.numel() else 0

    def prefix(ts):
        # for each threshold t of ts: the largest c in [0, hi - lo] with
        # qb * Qs[lo + c - 1] > t (Qs descending in a segment); both thresholds bisect
        # together, one set of tensor operations per step
        tt = torch.tensor(ts, dtype=Qs.dtype, device=dev)[:, None]
        a = torch.zeros((len(ts), lo.numel()), dtype=lo.dtype, device=dev)
        b = (hi - lo).expand(len(ts), -1).clone()
        for _ in range(nbits):
            mid = (a + b + 1) // 2
            ok = (mid > 0) & (qb * Qs[(lo + mid - 1).clamp(0, max(npair - 1, 0))] > tt)
            a = torch.where(ok, mid, a)
            b = torch.where(ok, b, mid - 1)
        return a

    if thr32 > 0:
        c, c32 = prefix([thr, thr32])
        c32 = torch.minimum(c32, c)
    else:
        c = prefix([thr])[0]
        c32 = c
    same = kk == kb
    r = pos - lo
    cnt = torch.where(same, torch.minimum(r + 1, c), c)
    diag = (same & (c <= r)).to(torch.int64)
    c64 = torch.minimum(cnt, c32)
    cls_row = class_table[kb, kk]
    bra = o[pos]
    plan = []
    ncls = int(class_table.max()) + 1 if class_table.numel() else 0
    for part, n, qs, dg in (("64", c64 + diag, lo, diag), ("32", cnt - c64, lo + c64, torch.zeros_like(diag))):
        # rows grouped by class (a stable sort keeps each class's rows in order), the
        # class sizes read back once per part
        key = torch.where(n > 0, cls_row, torch.full_like(cls_row, ncls))
        order = torch.sort(key, stable=True).indices
        counts = torch.bincount(key, minlength=ncls + 1)[:ncls].tolist()
        start = 0
        for cls, c in enumerate(counts):
            if c == 0:
                continue
            sel = order[start:start + c]
            start += c
            off = torch.cat([torch.zeros(1, dtype=torch.int64, device=dev), torch.cumsum(n[sel], 0)])
            plan.append((cls, part, bra[sel], off, qs[sel], dg[sel]))
    return plan, o


class GpuEngine:
    """Integrals of one molecule on one GPU.

    precision: "fp64" -- every quartet in double precision;
               "mixed" -- quartets with Schwarz bound Q_ab Q_cd < ``fp32_below`` in
               single precision, the rest and all accumulation in double.
    """

    def __init__(self, mol, device="cuda", precision="fp64", fp32_below=1e-4, threshold=INTEGRAL_THRESHOLD):
        if not torch.cuda.is_available():
            raise _lib.PcgError("pychem_gb300 needs a CUDA device")
        self.mol = mol
        self.dev = torch.device(device)
        self.precision = precision
        self.fp32_below = fp32_below if precision == "mixed" else 0.0
        self.threshold = threshold
        _lib.call("pcg_device_init")
        self._upload_basis()
        self._build_pairs()
        self.S = self.H = None
        self.classes = {}
        self.stats = {}

    # ---------------------------------------------------------------------------------
    def _t(self, a, dtype=None):
        return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype).to(self.dev)

    def _upload_basis(self):
        a = self.mol.arrays()
        self.h_basis = a
        self.d = {k: self._t(v) for k, v in a.items()}
        b = BasisT()
        b.nshell = len(a["sh_l"]); b.nprim = len(a["pr_exp"]); b.natom = len(a["at_z"]); b.nbf = self.mol.NOrbitals
        for k in ("sh_l", "sh_nprim", "sh_prim", "sh_ao", "sh_atom", "sh_xyz", "pr_exp", "pr_cc", "at_xyz", "at_z"):
            setattr(b, k, self.d[k].data_ptr())
        b.ld = self.mol.NOrbitals
        self.basis_t = b
        self.nbf = self.mol.NOrbitals

    def _build_pairs(self):
        """All shell pairs a <= b, oriented so that l_A >= l_B (their kinds are set by
        compute_pair_data)."""
        a = self.h_basis
        ns = len(a["sh_l"])
        ia, ib = np.triu_indices(ns)
        la, lb = a["sh_l"][ia], a["sh_l"][ib]
        swap = lb > la
        A = np.where(swap, ib, ia).astype(np.int32)
        B = np.where(swap, ia, ib).astype(np.int32)
        self._finish_pairs(A, B)

    def _finish_pairs(self, A, B):
        a = self.h_basis
        nA, nB = a["sh_nprim"][A], a["sh_nprim"][B]
        npp = (nA * nB).astype(np.int32)
        ppoff = np.concatenate([[0], np.cumsum(npp)[:-1]]).astype(np.int32)
        self.h_pairs = dict(A=A, B=B, npp=npp, ppoff=ppoff, lA=a["sh_l"][A], lB=a["sh_l"][B], nA=nA, nB=nB)
        self.npair = len(A)
        tot = int(npp.sum())
        dv = self.dev
        # every primitive pair (pcg_pair_data writes these) ...
        self.pd_full = dict(ppoff=self._t(ppoff), npp=self._t(npp),
                            zeta=torch.empty(tot, dtype=torch.float64, device=dv),
                            P=torch.empty(tot * 3, dtype=torch.float64, device=dv),
                            PA=torch.empty(tot * 3, dtype=torch.float64, device=dv),
                            K=torch.empty(tot, dtype=torch.float64, device=dv),
                            Kf=torch.empty(tot, dtype=torch.float32, device=dv),
                            oo2z=torch.empty(tot, dtype=torch.float64, device=dv))
        # ... and the kept ones, which the ERI kernels read (filled by compute_pair_data)
        self.pd = dict(A=self._t(A), B=self._t(B), AB=torch.empty(self.npair * 3, dtype=torch.float64, device=dv),
                       ao4=torch.empty(self.npair * 4, dtype=torch.int32, device=dv))
        self.pairs_t = PairsT()
        self.compute_pair_data()

    # primitive pairs with |K_p| max|K| below this are dropped (0 keeps all): every
    # primitive-quartet term of an integral carries the factor K_P K_Q
    prim_tau = 1e-20

    def _set_pairs_t(self):
        p, t = self.pd, self.pairs_t
        t.npair = self.npair
        t.npp = int(p["zeta"].numel())
        for k, f in (("A", "A"), ("B", "B"), ("ppoff", "ppoff"), ("npp", "npp_of"), ("AB", "AB"), ("zeta", "zeta"),
                     ("P", "P"), ("PA", "PA"), ("K", "K"), ("oo2z", "oo2z"), ("Kf", "Kf"), ("ao4", "ao4"), ("pf8", "pf8")):
            setattr(t, f, p[k].data_ptr())

    def _compact_primitives(self):
        """Keep the primitive pairs with |K_p| max|K| >= prim_tau, pair by pair (each
        pair's kept primitives stay contiguous), and re-derive the pair kinds
        (pair class, kept primitive pairs) that bucket the quartets."""
        f, p = self.pd_full, self.pd
        keep = f["K"].abs() * f["K"].abs().max() >= self.prim_tau
        idx = keep.nonzero().squeeze(1)
        cs = torch.cat([torch.zeros(1, dtype=torch.int64, device=self.dev), torch.cumsum(keep.to(torch.int64), 0)])
        start = f["ppoff"].to(torch.int64)
        cnt = cs[start + f["npp"].to(torch.int64)] - cs[start]
        p["ppoff"] = cs[start].to(torch.int32)
        p["npp"] = cnt.to(torch.int32)
        p["zeta"] = f["zeta"][idx]
        p["K"] = f["K"][idx]
        p["Kf"] = f["Kf"][idx]
        p["oo2z"] = f["oo2z"][idx]
        p["P"] = f["P"].view(-1, 3)[idx].reshape(-1)
        p["PA"] = f["PA"].view(-1, 3)[idx].reshape(-1)
        p["pf8"] = torch.empty(idx.numel() * 8, dtype=torch.float32, device=self.dev)
        # pair kinds ordered by (pair class, kept primitive pairs)
        npp = cnt.cpu().numpy().astype(np.int64)
        self.h_npp = npp
        pc = pair_class(self.h_pairs["lA"], self.h_pairs["lB"]).astype(np.int64)
        mb = int(npp.max()) + 1
        uniq, inv = np.unique(pc * mb + npp, return_inverse=True)
        self.kinds = [(int(c // mb), int(c % mb)) for c in uniq]
        self.pair_kind = np.asarray(inv).ravel().astype(np.int32)

    def compute_pair_data(self):
        """Primitive-pair data of every pair, the negligible primitive pairs dropped
        (_compact_primitives), the per-pair AO table and the packed FP32 primitive-pair
        table, from the device-resident shells."""
        p, f = self.pd, self.pd_full
        _lib.call("pcg_pair_data", ctypes.byref(self.basis_t), self.npair, _ptr(p["A"]), _ptr(p["B"]), _ptr(f["ppoff"]),
                  _ptr(p["AB"]), _ptr(f["zeta"]), _ptr(f["P"]), _ptr(f["PA"]), _ptr(f["K"]), _ptr(f["Kf"]),
                  _ptr(f["oo2z"]), _stream())
        self._compact_primitives()
        _lib.call("pcg_pair_ao", ctypes.byref(self.basis_t), self.npair, _ptr(p["A"]), _ptr(p["B"]), _ptr(p["ao4"]),
                  _stream())
        _lib.call("pcg_pair_data_f32", int(p["zeta"].numel()), _ptr(p["zeta"]), _ptr(p["PA"]), _ptr(p["oo2z"]),
                  _ptr(p["Kf"]), _ptr(p["pf8"]), _stream())
        self._set_pairs_t()

    # ---------------------------------------------------------------------------------
    def one_electron(self):
        n = self.nbf
        S = torch.zeros(n, n, dtype=torch.float64, device=self.dev)
        H = torch.zeros(n, n, dtype=torch.float64, device=self.dev)
        _lib.call("pcg_one_electron", ctypes.byref(self.basis_t), self.npair, _ptr(self.pd["A"]), _ptr(self.pd["B"]),
                  _ptr(S), _ptr(H), _stream())
        self.S, self.H = S, H
        return S, H

    # two-electron operator: None for 1/r12, S >= 0 for j0(S r12) (electron scattering,
    # Methods/properties.py:20-23); schwarz(), build_tasks() and compute_eris() follow it
    scattering = None

    def _eri(self, cls, tasks, ntask, store, fp32, pairs=None):
        pairs = self.pairs_t if pairs is None else pairs
        if self.scattering is not None:
            if fp32:
                raise ValueError("scattering integrals are FP64 only")
            _lib.call("pcg_scattering_class", cls, ctypes.byref(self.basis_t), ctypes.byref(pairs),
                      _ptr(tasks), ntask, float(self.scattering), _ptr(store), _stream())
            return
        _lib.call("pcg_eri_class", cls, ctypes.byref(self.basis_t), ctypes.byref(pairs), _ptr(tasks), ntask,
                  _ptr(store), 1 if fp32 else 0, _stream())

    # bra primitive pairs per task in the Schwarz pass
    schwarz_slice = 4

    def _sliced_pairs(self, ids, nslice):
        """A pair table of len(ids) * nslice bra slices -- slice s of pair k covers its
        kept primitive pairs [s * schwarz_slice, (s + 1) * schwarz_slice) -- followed by
        the len(ids) whole pairs, sharing the primitive arrays (device tensors kept in
        the returned tuple)."""
        p, ch = self.pd, self.schwarz_slice
        idt = torch.as_tensor(ids, dtype=torch.int64).to(self.dev)
        sl = torch.arange(nslice, dtype=torch.int64, device=self.dev)
        rep = lambda x: torch.cat([x.repeat_interleave(nslice, dim=0), x])
        off, cnt = p["ppoff"][idt].to(torch.int64), p["npp"][idt].to(torch.int64)
        s_off = (off[:, None] + sl[None, :] * ch).reshape(-1)
        s_cnt = (cnt[:, None] - sl[None, :] * ch).clamp(0, ch).reshape(-1)
        keep = dict(A=rep(p["A"][idt]).contiguous(), B=rep(p["B"][idt]).contiguous(),
                    AB=rep(p["AB"].view(-1, 3)[idt]).reshape(-1).contiguous(),
                    ppoff=torch.cat([s_off, off]).to(torch.int32), npp=torch.cat([s_cnt, cnt]).to(torch.int32))
        t = PairsT()
        ctypes.memmove(ctypes.addressof(t), ctypes.addressof(self.pairs_t), ctypes.sizeof(PairsT))
        t.npair = len(ids) * (nslice + 1)
        for k, f in (("A", "A"), ("B", "B"), ("ppoff", "ppoff"), ("npp", "npp_of"), ("AB", "AB")):
            setattr(t, f, keep[k].data_ptr())
        t.ao4 = None
        return t, keep

    def schwarz(self):
        """Q[pair] = sqrt(max (mn|mn)) over the diagonal quartets (ab|ab).  A diagonal
        quartet of many primitive pairs (the oxygen 1s pair: 36, so 1,296 primitive
        quartets) would run long on one thread, so the bra's kept primitive pairs are
        split into slices of schwarz_slice, each slice one task against the whole ket
        pair; the slices' integrals (linear in the primitive sum) are added in a fixed
        order before the maximum."""
        Q = torch.zeros(self.npair, dtype=torch.float64, device=self.dev)
        pc = pair_class(self.h_pairs["lA"], self.h_pairs["lB"])
        self.diag_blocks = {}
        npp = self.h_npp
        for c in np.unique(pc):
            ids = np.nonzero(pc == c)[0].astype(np.int32)
            # heaviest pairs first: the warps run uniform primitive loops and the long
            # quartets start early
            ids = ids[np.argsort(-npp[ids], kind="stable")]
            la, lb = int(self.h_pairs["lA"][ids[0]]), int(self.h_pairs["lB"][ids[0]])
            cls = _lib.load().pcg_eri_class_id(la, lb, la, lb)
            m = len(ids)
            nout = _lib.load().pcg_eri_class_nout(cls)
            nslice = 1 if self.scattering is not None else max(1, -(-int(npp[ids].max()) // self.schwarz_slice))
            if nslice == 1:
                tasks = self._t(np.stack([ids, ids], axis=1))
                store = torch.empty(nout * m, dtype=torch.float64, device=self.dev)
                self._eri(cls, tasks, m, store, False)
            else:
                pairs, keep = self._sliced_pairs(ids, nslice)
                vt = np.stack([np.arange(m * nslice), m * nslice + np.repeat(np.arange(m), nslice)], axis=1)
                vtasks = self._t(vt.astype(np.int32))
                part = torch.empty(nout * m * nslice, dtype=torch.float64, device=self.dev)
                self._eri(cls, vtasks, m * nslice, part, False, pairs=pairs)
                store = part.view(nout, m, nslice).sum(dim=2).contiguous()
                tasks = self._t(np.stack([ids, ids], axis=1))
                del keep
            _lib.call("pcg_schwarz_class", cls, _ptr(tasks), m, _ptr(store), _ptr(Q), _stream())
        self.Q = Q
        return Q

    # ---------------------------------------------------------------------------------
    def _pair_molecule(self):
        """Molecule index of every shell pair (device int64) and the molecule count."""
        return torch.zeros(self.npair, dtype=torch.int64, device=self.dev), 1

    def build_tasks(self):
        """Screened canonical quartet lists per class and precision part, planned on the
        GPU by plan_quartets() and expanded by the library (one launch per class and
        part)."""
        dev = self.dev
        nk = len(self.kinds)
        order = np.argsort(self.pair_kind, kind="stable")
        first = order[np.searchsorted(self.pair_kind[order], np.arange(nk))]
        kl = np.stack([self.h_pairs["lA"][first], self.h_pairs["lB"][first]], axis=1)
        ct = np.full((nk, nk), -1, dtype=np.int64)
        lib = _lib.load()
        for i in range(nk):
            for j in range(i + 1):
                ct[i, j] = lib.pcg_eri_class_id(int(kl[i, 0]), int(kl[i, 1]), int(kl[j, 0]), int(kl[j, 1]))
        mol, nmol = self._pair_molecule()
        work = torch.as_tensor([k[1] for k in self.kinds], dtype=torch.int64, device=dev)
        plan, ket_list = plan_quartets(self.Q, torch.as_tensor(self.pair_kind, dtype=torch.int64, device=dev), mol,
                                       nmol, torch.as_tensor(ct, device=dev), float(self.threshold),
                                       float(self.fp32_below), kind_work=work)
        totals = torch.stack([x[3][-1] for x in plan]).cpu().tolist() if plan else []
        ket32 = ket_list.to(torch.int32)
        self.classes = {}
        for (cls, part, bra, off, qs, dg), total in zip(plan, totals):
            tasks = torch.empty(int(total) * 2, dtype=torch.int32, device=dev)
            # named so that the int32 copies outlive the launch that reads them
            bra32, qs32, dg32 = bra.to(torch.int32), qs.to(torch.int32), dg.to(torch.int32)
            _lib.call("pcg_expand_tasks", bra.numel(), _ptr(bra32), _ptr(ket32), _ptr(off), _ptr(qs32), _ptr(dg32),
                      int(total), _ptr(tasks), _stream())
            self.classes.setdefault(cls, {})[part] = (tasks, int(total))
        self.classes = dict(sorted(self.classes.items()))
        self._task_stats()
        return self.classes

    @property
    def prim_quartets(self):
        """Primitive quartets per (class, part) of the current task lists (for the
        algorithmic flop count), computed on first use after build_tasks."""
        if self._prim_quartets is None:
            self._prim_quartets = {}
            npp = self.pd["npp"].to(torch.int64)
            for cls, rec in self.classes.items():
                for part, (tasks, n) in rec.items():
                    tv = tasks.view(n, 2).to(torch.int64)
                    self._prim_quartets[(cls, part)] = (npp[tv[:, 0]] * npp[tv[:, 1]]).sum()
        return self._prim_quartets

    _prim_quartets = None

    def _task_stats(self):
        nq64 = sum(rec["64"][1] for rec in self.classes.values() if "64" in rec)
        nq32 = sum(rec["32"][1] for rec in self.classes.values() if "32" in rec)
        self._prim_quartets = None
        self.stats["quartets_fp64"] = nq64
        self.stats["quartets_fp32"] = nq32
        self.stats["quartets"] = nq64 + nq32

    def compute_eris(self):
        """Compute every screened quartet block into the in-core class stores."""
        self.stores = {}
        for cls, rec in self.classes.items():
            nout = _lib.load().pcg_eri_class_nout(cls)
            for part, (tasks, n) in rec.items():
                store = torch.empty(nout * n, dtype=torch.float64, device=self.dev)
                self._eri(cls, tasks, n, store, part == "32")
                self.stores[(cls, part)] = store
        return self.stores

    def prepare(self, recompute_pairs=False):
        """One-electron matrices, Schwarz factors, task lists and ERI store."""
        if recompute_pairs:
            self.compute_pair_data()
        self.one_electron()
        self.schwarz()
        self.build_tasks()
        self.compute_eris()
        return self

    # ---------------------------------------------------------------------------------
    def fock(self, D, out=None, G=None):
        """Closed-shell F = H + 2J[D] - K[D] for the alpha density D (nbf x nbf)."""
        n = self.nbf
        if G is None:
            G = torch.zeros(n, n, dtype=torch.float64, device=self.dev)
        else:
            G.zero_()
        D = D.contiguous()
        for cls, rec in self.classes.items():
            for part, (tasks, ntask) in rec.items():
                _lib.call("pcg_digest_class", cls, ctypes.byref(self.basis_t), ctypes.byref(self.pairs_t), _ptr(tasks),
                          ntask, _ptr(self.stores[(cls, part)]), _ptr(D), _ptr(G), _stream())
        F = out if out is not None else torch.empty(n, n, dtype=torch.float64, device=self.dev)
        _lib.call("pcg_fock_build", n, _ptr(self.H), _ptr(G), _ptr(F), _stream())
        return F

    def fock_u(self, Da, Db):
        """Unrestricted Fock matrices F_s = H + J[D_a + D_b] - K[D_s] (nbf x nbf each)."""
        n = self.nbf
        G = torch.zeros(3, n, n, dtype=torch.float64, device=self.dev)
        Da, Db = Da.contiguous(), Db.contiguous()
        for cls, rec in self.classes.items():
            for part, (tasks, ntask) in rec.items():
                _lib.call("pcg_digest_class_u", cls, ctypes.byref(self.basis_t), ctypes.byref(self.pairs_t),
                          _ptr(tasks), ntask, _ptr(self.stores[(cls, part)]), _ptr(Da), _ptr(Db), _ptr(G[0]),
                          _ptr(G[1]), _ptr(G[2]), _stream())
        Ga, Gb = G[0] + G[1], G[0] + G[2]
        return self.H + 0.5 * (Ga + Ga.T), self.H + 0.5 * (Gb + Gb.T)

    def coulomb_exchange(self, W):
        """J[W] and K[W] for general (not necessarily symmetric) co-densities W of shape
        (nd, nbf, nbf): J_ab = sum_cd (ab|cd) W_cd, K_ad = sum_bc (ab|cd) W_cb
        (Methods/hartree_fock.py:345-347, applied by Methods/noci.py:261-318).

        One pcg_digest_class_co launch per class part digests every density (blockIdx.y
        selects it).  Per unique quartet the digestion accumulates one orientation of
        each exchange block (G[M]_ad from M_bc and so on); the kernel adds G[W^T] and
        G[W]^T, which together hold all eight index permutations: K[W] = -GK/2.  The
        Coulomb buffer sees (W + W^T)/2, all that J depends on: J = (GJ + GJ^T)/4."""
        W = W.contiguous()
        nd = W.shape[0]
        GJ = torch.zeros_like(W)
        GK = torch.zeros_like(W)
        for cls, rec in self.classes.items():
            for part, (tasks, ntask) in rec.items():
                _lib.call("pcg_digest_class_co", cls, ctypes.byref(self.basis_t), ctypes.byref(self.pairs_t),
                          _ptr(tasks), ntask, _ptr(self.stores[(cls, part)]), nd, _ptr(W), _ptr(GJ), _ptr(GK),
                          _stream())
        return 0.25 * (GJ + GJ.transpose(1, 2)), -0.5 * GK

    def stored_pair_map(self):
        """(map, count): for every AO pair a >= b, at pair(a, b) = a(a+1)/2 + b, its row
        in a compact pair-packed tensor, or -1 when its shell pair is in no stored
        quartet but its own diagonal one (ab|ab) -- the quartet upstream always
        computes, whose value is below (1e-8 / max Q)^2 ~ 1e-16 when the pair fails
        every Schwarz test, and which MP2 then leaves out; rows follow pair order.  On
        a 16-water cluster 56 % of the AO pairs have rows."""
        n = self.nbf
        nao2 = n * (n + 1) // 2
        if getattr(self, "_ao_shell_pair", None) is None or self._ao_shell_pair[0] is not self.h_pairs:
            # the shell pair of every AO pair a >= b
            a, hp = self.h_basis, self.h_pairs
            ao, dim = a["sh_ao"].astype(np.int64), 2 * a["sh_l"].astype(np.int64) + 1
            i, j = np.divmod(np.arange(25), 5)
            fa = ao[hp["A"]][:, None] + i[None, :]
            fb = ao[hp["B"]][:, None] + j[None, :]
            ok = (i[None, :] < dim[hp["A"]][:, None]) & (j[None, :] < dim[hp["B"]][:, None])
            hi, lo = np.maximum(fa, fb), np.minimum(fa, fb)
            sp = np.empty(nao2, dtype=np.int64)
            sp[(hi * (hi + 1) // 2 + lo)[ok]] = np.broadcast_to(np.arange(self.npair)[:, None], ok.shape)[ok]
            self._ao_shell_pair = (self.h_pairs, torch.as_tensor(sp, device=self.dev))
        # shell pairs in some off-diagonal stored quartet (pcg_mark_pairs), no host round trip
        used = torch.zeros(self.npair, dtype=torch.bool, device=self.dev)
        for rec in self.classes.values():
            for tasks, ntask in rec.values():
                _lib.call("pcg_mark_pairs", _ptr(tasks), ntask, _ptr(used), _stream())
        flag = used[self._ao_shell_pair[1]]
        rank = torch.cumsum(flag, 0, dtype=torch.int32)
        pmap = torch.where(flag, rank - 1, -1).to(torch.int32)
        return pmap, int(rank[-1])

    def dense_eri_pairs(self, compact=False):
        """The dense tensor with the bra pair packed: E[pair(a, b)][c][d], a >= b,
        pair(a, b) = a(a+1)/2 + b (nbf(nbf+1)/2 x nbf x nbf), zero where screened out.
        compact=True keeps only the AO pairs with rows in stored_pair_map and returns
        (E (count x nbf x nbf), map, count); it goes through the count x count symmetric
        pair matrix (two scattered stores per stored element, then one coalesced unpack)."""
        n = self.nbf
        if compact:
            # the rows x rows symmetric pair matrix, then its columns unpacked to (c, d)
            pmap, rows = self.stored_pair_map()
            M = torch.zeros(rows * rows, dtype=torch.float64, device=self.dev)
            for cls, rec in self.classes.items():
                for part, (tasks, ntask) in rec.items():
                    _lib.call("pcg_sym_pairs_class", cls, ctypes.byref(self.basis_t), ctypes.byref(self.pairs_t),
                              _ptr(tasks), ntask, _ptr(self.stores[(cls, part)]), _ptr(pmap), rows, _ptr(M),
                              _stream())
            E = torch.empty(rows, n, n, dtype=torch.float64, device=self.dev)
            _lib.call("pcg_unpack_pairs", rows, n, rows, _ptr(pair_colmap(n, pmap, self.dev)), _ptr(M), _ptr(E),
                      _stream())
            return E, pmap, rows
        pmap, rows = None, n * (n + 1) // 2
        E = torch.zeros(rows * n * n, dtype=torch.float64, device=self.dev)
        for cls, rec in self.classes.items():
            for part, (tasks, ntask) in rec.items():
                _lib.call("pcg_dense_pairs_class", cls, ctypes.byref(self.basis_t), ctypes.byref(self.pairs_t),
                          _ptr(tasks), ntask, _ptr(self.stores[(cls, part)]), _ptr(pmap), _ptr(E), _stream())
        E = E.view(rows, n, n)
        return (E, pmap, rows) if compact else E

    def prefetch_mp2_tensor(self):
        """Start dense_eri_pairs(compact=True) on a side stream -- it reads only the ERI
        store -- so that it runs beside the SCF (whose first iteration and final
        orbitals leave most SMs idle).  Returns ((E, map, rows), event): the tuple is
        for scf.rmp2(eri=...) once the current stream has waited for the event."""
        main = torch.cuda.current_stream(self.dev)
        if getattr(self, "_side", None) is None:
            self._side = torch.cuda.Stream(self.dev)
        side = self._side
        side.wait_stream(main)
        with torch.cuda.stream(side):
            E, pmap, rows = self.dense_eri_pairs(compact=True)
            ev = torch.cuda.Event()
            ev.record(side)
        E.record_stream(main)
        pmap.record_stream(main)
        return (E, pmap, rows), ev

    def dense_eri(self):
        """Dense nbf^4 tensor (8-fold symmetric fill), zero where screened out."""
        n = self.nbf
        eri = torch.zeros(n ** 4, dtype=torch.float64, device=self.dev)
        for cls, rec in self.classes.items():
            for part, (tasks, ntask) in rec.items():
                _lib.call("pcg_dense_class", cls, ctypes.byref(self.basis_t), ctypes.byref(self.pairs_t), _ptr(tasks),
                          ntask, _ptr(self.stores[(cls, part)]), _ptr(eri), _stream())
        return eri.view(n, n, n, n)
