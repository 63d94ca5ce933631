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
        """All shell pairs a <= b, oriented so that l_A >= l_B; kinds = (l_A, l_B, nA, nB)."""
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
        self.pd = dict(A=self._t(A), B=self._t(B), ppoff=self._t(ppoff), npp=self._t(npp),
                       AB=torch.empty(self.npair * 3, dtype=torch.float64, device=dv),
                       zeta=torch.empty(tot, dtype=torch.float64, device=dv),
                       P=torch.empty(tot * 3, dtype=torch.float64, device=dv),
                       PA=torch.empty(tot * 3, dtype=torch.float64, device=dv),
                       K=torch.empty(tot, dtype=torch.float64, device=dv),
                       Kf=torch.empty(tot, dtype=torch.float32, device=dv),
                       oo2z=torch.empty(tot, dtype=torch.float64, device=dv))
        p = self.pd
        t = PairsT()
        t.npair = self.npair; t.npp = tot
        for k, f in (("A", "A"), ("B", "B"), ("ppoff", "ppoff"), ("npp", "npp_of"), ("AB", "AB"), ("zeta", "zeta"),
                     ("P", "P"), ("PA", "PA"), ("K", "K"), ("oo2z", "oo2z"), ("Kf", "Kf")):
            setattr(t, f, p[k].data_ptr())
        self.pairs_t = t
        # pair kinds ordered by (pair class, nA, nB)
        keys = np.stack([pair_class(self.h_pairs["lA"], self.h_pairs["lB"]), nA, nB], axis=1)
        uniq = np.unique(keys, axis=0)
        order = np.lexsort((uniq[:, 2], uniq[:, 1], uniq[:, 0]))
        self.kinds = [tuple(int(x) for x in uniq[i]) for i in order]
        kind_index = {k: i for i, k in enumerate(self.kinds)}
        self.pair_kind = np.array([kind_index[tuple(int(x) for x in r)] for r in keys], dtype=np.int32)
        self.compute_pair_data()

    def compute_pair_data(self):
        """Primitive-pair data from the device-resident shells (one kernel)."""
        p = self.pd
        _lib.call("pcg_pair_data", ctypes.byref(self.basis_t), self.npair, _ptr(p["A"]), _ptr(p["B"]), _ptr(p["ppoff"]),
                  _ptr(p["AB"]), _ptr(p["zeta"]), _ptr(p["P"]), _ptr(p["PA"]), _ptr(p["K"]), _ptr(p["Kf"]),
                  _ptr(p["oo2z"]), _stream())

    # ---------------------------------------------------------------------------------
    def one_electron(self):
        n = self.nbf
        S = torch.zeros(n, n, dtype=torch.float64, device=self.dev)
        H = torch.zeros(n, n, dtype=torch.float64, device=self.dev)
        _lib.call("pcg_one_electron", ctypes.byref(self.basis_t), self.npair, _ptr(self.pd["A"]), _ptr(self.pd["B"]),
                  _ptr(S), _ptr(H), _stream())
        self.S, self.H = S, H
        return S, H

    def _eri(self, cls, tasks, ntask, store, fp32):
        _lib.call("pcg_eri_class", cls, ctypes.byref(self.basis_t), ctypes.byref(self.pairs_t), _ptr(tasks), ntask,
                  _ptr(store), 1 if fp32 else 0, _stream())

    def schwarz(self):
        """Q[pair] = sqrt(max (mn|mn)) over the diagonal quartets (ab|ab)."""
        Q = torch.zeros(self.npair, dtype=torch.float64, device=self.dev)
        pc = pair_class(self.h_pairs["lA"], self.h_pairs["lB"])
        self.diag_blocks = {}
        for c in np.unique(pc):
            ids = np.nonzero(pc == c)[0].astype(np.int32)
            la, lb = int(self.h_pairs["lA"][ids[0]]), int(self.h_pairs["lB"][ids[0]])
            cls = _lib.load().pcg_eri_class_id(la, lb, la, lb)
            tasks = self._t(np.stack([ids, ids], axis=1))
            nout = _lib.load().pcg_eri_class_nout(cls)
            store = torch.empty(nout * len(ids), dtype=torch.float64, device=self.dev)
            self._eri(cls, tasks, len(ids), store, False)
            _lib.call("pcg_schwarz_class", cls, _ptr(tasks), len(ids), _ptr(store), _ptr(Q), _stream())
        self.Q = Q
        return Q

    # ---------------------------------------------------------------------------------
    def build_tasks(self):
        """Screened canonical quartet lists per class (FP64 part and FP32 part)."""
        Qh = self.Q.cpu().numpy()
        thr, thr32 = self.threshold, self.fp32_below
        kp, ks = [], []   # per kind: pair ids sorted by Q desc, their Q
        for k in range(len(self.kinds)):
            ids = np.nonzero(self.pair_kind == k)[0]
            o = np.argsort(-Qh[ids], kind="stable")
            kp.append(ids[o].astype(np.int32))
            ks.append(Qh[ids[o]])
        self.kind_pairs_dev = [self._t(x) for x in kp]

        def prefix_count(Qr, Qk, t):
            # number of leading kets with Qr * Qk > t (Qk sorted descending)
            c = np.searchsorted(-Qk, -(t / np.maximum(Qr, 1e-300)), side="left")
            n = len(Qk)
            for _ in range(2):
                up = (c < n) & (Qr * Qk[np.minimum(c, n - 1)] > t)
                c = c + up
                dn = (c > 0) & ~(Qr * Qk[np.maximum(c - 1, 0)] > t)
                c = c - dn
            return c.astype(np.int64)

        per_class = {}
        nk = len(self.kinds)
        for kb in range(nk):
            for kk in range(kb + 1):
                pb, lab, lbb = self.kinds[kb][0], None, None
                bra_ids, ket_ids = kp[kb], kp[kk]
                if len(bra_ids) == 0 or len(ket_ids) == 0:
                    continue
                la, lb = int(self.h_pairs["lA"][bra_ids[0]]), int(self.h_pairs["lB"][bra_ids[0]])
                lc, ld = int(self.h_pairs["lA"][ket_ids[0]]), int(self.h_pairs["lB"][ket_ids[0]])
                cls = _lib.load().pcg_eri_class_id(la, lb, lc, ld)
                Qr, Qk = ks[kb], ks[kk]
                c = prefix_count(Qr, Qk, thr)
                c32 = prefix_count(Qr, Qk, thr32) if thr32 > 0 else np.full(len(Qr), len(Qk), dtype=np.int64)
                c32 = np.minimum(c32, c)
                if kb == kk:
                    r = np.arange(len(Qr), dtype=np.int64)
                    cnt = np.minimum(r + 1, c)
                    diag = (c <= r).astype(np.int32)
                    c64 = np.minimum(cnt, c32)
                else:
                    cnt = c
                    diag = np.zeros(len(Qr), dtype=np.int32)
                    c64 = c32
                n64 = c64 + diag
                n32 = cnt - c64
                entry = per_class.setdefault(cls, {"64": [], "32": []})
                entry["64"].append((kb, kk, n64, np.zeros(len(Qr), dtype=np.int32), diag))
                if n32.sum() > 0:
                    entry["32"].append((kb, kk, n32, c64.astype(np.int32), np.zeros(len(Qr), dtype=np.int32)))
        return self._expand(per_class)

    def _expand(self, per_class):
        """Materialise the per-bra (count, first ket, diagonal) bucket plans as int2
        task lists on the GPU, one per class and precision."""
        self.classes = {}
        nq64 = nq32 = 0
        for cls, entry in sorted(per_class.items()):
            rec = {}
            for part in ("64", "32"):
                buckets = entry[part]
                total = int(sum(int(b[2].sum()) for b in buckets))
                if total == 0:
                    continue
                tasks = torch.empty(total * 2, dtype=torch.int32, device=self.dev)
                pos = 0
                for (kb, kk, cnt, qstart, diag) in buckets:
                    ntask = int(cnt.sum())
                    if ntask == 0:
                        continue
                    off = np.concatenate([[0], np.cumsum(cnt)]).astype(np.int64)
                    d_off, d_qs, d_dg = self._t(off), self._t(qstart), self._t(diag)
                    sub = tasks[2 * pos:]
                    _lib.call("pcg_expand_tasks", len(cnt), _ptr(self.kind_pairs_dev[kb]), _ptr(self.kind_pairs_dev[kk]),
                              _ptr(d_off), _ptr(d_qs), _ptr(d_dg), ntask, _ptr(sub), _stream())
                    pos += ntask
                rec[part] = (tasks, total)
            self.classes[cls] = rec
            nq64 += rec.get("64", (None, 0))[1]
            nq32 += rec.get("32", (None, 0))[1]
        # primitive quartets per class and part (for the algorithmic flop count)
        self.prim_quartets = {}
        npp = self.pd["npp"].to(torch.int64)
        for cls, rec in self.classes.items():
            for part, (tasks, n) in rec.items():
                tv = tasks.view(n, 2).to(torch.int64)
                self.prim_quartets[(cls, part)] = (npp[tv[:, 0]] * npp[tv[:, 1]]).sum()
        self.stats["quartets_fp64"] = nq64
        self.stats["quartets_fp32"] = nq32
        self.stats["quartets"] = nq64 + nq32
        return self.classes

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

    def dense_eri(self):
        """Dense nbf^4 tensor (8-fold symmetric fill), zero where screened out."""
        n = self.nbf
        eri = torch.zeros(n ** 4, dtype=torch.float64, device=self.dev)
        for cls, rec in self.classes.items():
            for part, (tasks, ntask) in rec.items():
                _lib.call("pcg_dense_class", cls, ctypes.byref(self.basis_t), ctypes.byref(self.pairs_t), _ptr(tasks),
                          ntask, _ptr(self.stores[(cls, part)]), _ptr(eri), _stream())
        return eri.view(n, n, n, n)
