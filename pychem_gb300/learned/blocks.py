"""Atom-pair features and density blocks in the pair's bond frame (6-31G, H/C/N/O).

For an atom pair (i, j) the density block D[AO(i), AO(j)] is expressed in the local
frame whose z axis points from atom i to atom j (p orbitals rotate as vectors, s
orbitals are invariant): D_loc = T_i D T_j^T with T = blockdiag(1 per s shell, R per p
shell), R the rows (e_x, e_y, e_z).  A block of a pair in cylindrical symmetry has
only s-s, s-p_z, p_z-s, sigma (p_z-p_z) and pi (p_x-p_x = p_y-p_y) elements, so the
network predicts 29 numbers for heavy-heavy pairs, 10 for heavy-H and 4 for H-H
(slot masks select them), and blocks are rotated back with T_i^T D_loc T_j.

Features per ordered pair: one-hot element of i and of j (H, C, N, O) and 32
Gaussians exp(-(r - mu_k)^2 / (2 w^2)) of the distance in Angstrom, mu_k evenly
spaced over [0.5, 6] A with width w the spacing.  Pairs beyond 6 A are not predicted.
Every ordered pair (i, j) within the cutoff is used: its 29 off-diagonal slots
describe D[AO(i), AO(j)] (the two orders of a pair are averaged when a guess is
assembled) and its 18 further slots a symmetric cylindrical correction to atom i's
own block in the i->j frame; a guess's diagonal block of atom i is its free-atom (SAD)
block plus the rotated corrections summed over its neighbours j.
"""
import numpy as np
import torch

ELEMENTS = ["H", "C", "N", "O"]
EIDX = {e: k for k, e in enumerate(ELEMENTS)}
CUTOFF = 6.0
NG = 32
MU = np.linspace(0.5, 6.0, NG)
WIDTH = MU[1] - MU[0]
NFEAT = 8 + NG
NOFF = 29          # off-diagonal block slots
NDIAG = 18         # slots of the correction to atom i's own block from neighbour j
NPARAM = NOFF + NDIAG
TO_BOHR = 1.8897161646320724

HEAVY_SHELLS = [("s", 0), ("s", 1), ("p", 2), ("s", 5), ("p", 6)]
H_SHELLS = [("s", 0), ("s", 1)]


def shells_of(sym):
    return H_SHELLS if sym == "H" else HEAVY_SHELLS


def nao_of(sym):
    return 2 if sym == "H" else 9


def slots(ti, tj):
    """Parameter slots of a pair type ('H' or 'X' for each atom)."""
    si = H_SHELLS if ti == "H" else HEAVY_SHELLS
    sj = H_SHELLS if tj == "H" else HEAVY_SHELLS
    out = []
    for a, ao in si:
        for b, bo in sj:
            if a == "s" and b == "s":
                out.append(("ss", ao, bo))
            elif a == "s":
                out.append(("sp", ao, bo))
            elif b == "s":
                out.append(("ps", ao, bo))
            else:
                out.append(("pps", ao, bo))
                out.append(("ppp", ao, bo))
    return out


# the order gives the pair-type index tc = 2 [i is H] + [j is H]
TYPES = {("X", "X"): slots("X", "X"), ("X", "H"): slots("X", "H"), ("H", "X"): slots("H", "X"),
         ("H", "H"): slots("H", "H")}


def diag_slots(ti):
    """Symmetric cylindrical corrections to the block of atom i in the i->j frame."""
    sh = H_SHELLS if ti == "H" else HEAVY_SHELLS
    out = []
    for x in range(len(sh)):
        for y in range(x, len(sh)):
            (a, ao), (b, bo) = sh[x], sh[y]
            if a == "s" and b == "s":
                out.append(("ss", ao, bo))
            elif a == "s" or b == "s":
                so, po = (ao, bo) if a == "s" else (bo, ao)
                out.append(("sp", so, po))
            else:
                out.append(("pps", ao, bo))
                out.append(("ppp", ao, bo))
    return out


DIAG = {"X": diag_slots("X"), "H": diag_slots("H")}
assert len(DIAG["X"]) == NDIAG


def frames(vec):
    """Rows (e_x, e_y, e_z) with e_z along vec (P, 3) -> (P, 3, 3)."""
    ez = vec / vec.norm(dim=-1, keepdim=True)
    ax = torch.zeros_like(ez)
    ax.scatter_(1, ez.abs().argmin(dim=1, keepdim=True), 1.0)
    ex = ax - (ax * ez).sum(-1, keepdim=True) * ez
    ex = ex / ex.norm(dim=-1, keepdim=True)
    ey = torch.cross(ez, ex, dim=-1)
    return torch.stack([ex, ey, ez], dim=1)


def _T(R, shells, n):
    P = R.shape[0]
    T = torch.zeros(P, n, n, dtype=R.dtype, device=R.device)
    for kind, o in shells:
        if kind == "s":
            T[:, o, o] = 1.0
        else:
            T[:, o:o + 3, o:o + 3] = R
    return T


def params_from_blocks(blk, R, ti, tj):
    """(P, ni, nj) global blocks -> (P, NPARAM) slot values and mask."""
    ni, nj = (2 if ti == "H" else 9), (2 if tj == "H" else 9)
    loc = _T(R, shells_of("H" if ti == "H" else "C"), ni) @ blk @ _T(R, shells_of("H" if tj == "H" else "C"), nj).transpose(1, 2)
    P = blk.shape[0]
    out = torch.zeros(P, NOFF, dtype=blk.dtype, device=blk.device)
    mask = torch.zeros(NOFF, dtype=blk.dtype, device=blk.device)
    for k, (kind, a, b) in enumerate(TYPES[(ti, tj)]):
        if kind == "ss":
            out[:, k] = loc[:, a, b]
        elif kind == "sp":
            out[:, k] = loc[:, a, b + 2]
        elif kind == "ps":
            out[:, k] = loc[:, a + 2, b]
        elif kind == "pps":
            out[:, k] = loc[:, a + 2, b + 2]
        else:
            out[:, k] = 0.5 * (loc[:, a, b] + loc[:, a + 1, b + 1])
        mask[k] = 1.0
    return out, mask


def _put(E, k, a, b, sym):
    E[k, a, b] = 1.0
    if sym:
        E[k, b, a] = 1.0


def off_basis(ti, tj):
    """(NOFF, ni, nj) local-frame matrices: a block's local form is sum_k par_k E_k."""
    ni, nj = nao_of(ti), nao_of(tj)
    E = torch.zeros(NOFF, ni, nj, dtype=torch.float64)
    for k, (kind, a, b) in enumerate(TYPES[(ti, tj)]):
        if kind == "ss":
            E[k, a, b] = 1.0
        elif kind == "sp":
            E[k, a, b + 2] = 1.0
        elif kind == "ps":
            E[k, a + 2, b] = 1.0
        elif kind == "pps":
            E[k, a + 2, b + 2] = 1.0
        else:
            E[k, a, b] = E[k, a + 1, b + 1] = 1.0
    return E


def diag_basis(ti):
    """(NDIAG, ni, ni) symmetric local-frame matrices of the diagonal corrections."""
    ni = nao_of(ti)
    E = torch.zeros(NDIAG, ni, ni, dtype=torch.float64)
    for k, (kind, a, b) in enumerate(DIAG[ti]):
        if kind == "ss":
            _put(E, k, a, b, True)
        elif kind == "sp":
            _put(E, k, a, b + 2, True)
        elif kind == "pps":
            _put(E, k, a + 2, b + 2, True)
        else:
            _put(E, k, a, b, True)
            _put(E, k, a + 1, b + 1, True)
    return E


_BASIS_CACHE = {}


def _basis(key, dtype, device):
    k = (key, dtype, str(device))
    if k not in _BASIS_CACHE:
        E = diag_basis(key) if isinstance(key, str) else off_basis(*key)
        _BASIS_CACHE[k] = E.to(dtype=dtype, device=device)
    return _BASIS_CACHE[k]


def _Tmat(R, t):
    return _T(R, shells_of("H" if t == "H" else "C"), nao_of(t))


def diag_from_params(par, R, ti):
    """(P, NDIAG) corrections -> (P, ni, ni) symmetric global-frame blocks of atom i."""
    loc = torch.einsum("pk,kab->pab", par, _basis(ti, par.dtype, par.device))
    T = _Tmat(R.to(par.dtype), ti)
    return T.transpose(1, 2) @ loc @ T


def blocks_from_params(par, R, ti, tj):
    """(P, NOFF) slot values -> (P, ni, nj) global-frame blocks D[AO(i), AO(j)]."""
    loc = torch.einsum("pk,kab->pab", par, _basis((ti, tj), par.dtype, par.device))
    R = R.to(par.dtype)
    return _Tmat(R, ti).transpose(1, 2) @ loc @ _Tmat(R, tj)


ZIDX = torch.full((10,), -1, dtype=torch.int64)
ZIDX[1], ZIDX[6], ZIDX[7], ZIDX[8] = 0, 1, 2, 3


def pairs(at, device):
    """All ordered atom pairs (i, j), i != j, within the cutoff, from an atom table
    (mol, ao0, z, xyz [bohr], atom0, nat per molecule), built with tensor operations on
    `device`, ordered by molecule.  Returns tensors mol, gi, gj (atoms' table rows),
    ao_i, ao_j, ei, ej (element indices), r [A], vec = R_j - R_i [bohr] and tc, the
    pair type's index in TYPES."""
    nat = torch.as_tensor(at["nat"], device=device)
    nb, amax = nat.numel(), int(nat.max())
    mol = torch.as_tensor(at["mol"], device=device)
    N = mol.numel()
    z = torch.as_tensor(np.rint(at["z"]).astype(np.int64), device=device)
    if int(z.max()) >= ZIDX.numel() or bool((ZIDX.to(device)[z] < 0).any()):
        raise ValueError("the learned guess covers H, C, N and O only")
    eidx = ZIDX.to(device)[z]
    ao0 = torch.as_tensor(at["ao0"], device=device)
    loc = torch.arange(N, device=device) - torch.as_tensor(at["atom0"], device=device)[mol]
    idx = torch.full((nb, amax), -1, dtype=torch.int64, device=device)
    idx[mol, loc] = torch.arange(N, device=device)
    xyz = torch.zeros(nb, amax, 3, dtype=torch.float64, device=device)
    xyz[mol, loc] = torch.as_tensor(at["xyz"], dtype=torch.float64, device=device)
    vec = xyz[:, None, :, :] - xyz[:, :, None, :]
    r = torch.linalg.vector_norm(vec, dim=-1) / TO_BOHR
    valid = idx >= 0
    eye = torch.eye(amax, dtype=torch.bool, device=device)
    keep = valid[:, :, None] & valid[:, None, :] & ~eye[None] & (r <= CUTOFF)
    m, i, j = keep.nonzero(as_tuple=True)
    gi, gj = idx[m, i], idx[m, j]
    ei, ej = eidx[gi], eidx[gj]
    tc = 2 * (ei == 0).to(torch.int64) + (ej == 0).to(torch.int64)
    return dict(mol=m, gi=gi, gj=gj, ao_i=ao0[gi], ao_j=ao0[gj], ei=ei, ej=ej, r=r[m, i, j], vec=vec[m, i, j], tc=tc)


def features(pl, device):
    ei = torch.as_tensor(pl["ei"], device=device)
    ej = torch.as_tensor(pl["ej"], device=device)
    r = torch.as_tensor(pl["r"], dtype=torch.float32, device=device)
    P = r.numel()
    X = torch.zeros(P, NFEAT, dtype=torch.float32, device=device)
    X[torch.arange(P, device=device), ei] = 1.0
    X[torch.arange(P, device=device), 4 + ej] = 1.0
    mu = torch.as_tensor(MU, dtype=torch.float32, device=device)
    X[:, 8:] = torch.exp(-((r.unsqueeze(1) - mu) ** 2) / (2.0 * WIDTH ** 2))
    return X


def gather_blocks(D, pl, t):
    ni, nj = (2 if t[0] == "H" else 9), (2 if t[1] == "H" else 9)
    dev = D.device
    m = torch.as_tensor(pl["mol"], device=dev)[:, None, None]
    ai = torch.as_tensor(pl["ao_i"], device=dev)[:, None, None] + torch.arange(ni, device=dev)[None, :, None]
    aj = torch.as_tensor(pl["ao_j"], device=dev)[:, None, None] + torch.arange(nj, device=dev)[None, None, :]
    return D[m, ai, aj]
