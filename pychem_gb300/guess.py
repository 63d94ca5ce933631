"""Initial densities for the SCF.

* core: eigenvectors of the core Hamiltonian (upstream ``hartree_fock.py:55-57``).
* sad: superposition of atomic densities.  Upstream accepts ``SCF_Guess = SAD`` in its
  input parser (``Util/structures.py:211``) but never implements it; here each element
  gets a spherically averaged fractional-occupation SCF in the molecule's basis (every
  orbital of the partially filled level carries the same fraction), computed once per
  (element, basis) on the GPU and cached, and the molecular guess is the block-diagonal
  sum of the atomic alpha densities.
"""
import torch

from . import eigen

_ATOM_CACHE = {}


def _fractional_occupations(eps, nelec_alpha, degeneracy_tol=1e-3):
    order = torch.argsort(eps)
    e = eps[order]
    f = torch.zeros_like(e)
    left = float(nelec_alpha)
    i, n = 0, len(e)
    while left > 1e-12 and i < n:
        j = i + 1
        while j < n and float(e[j] - e[i]) < degeneracy_tol:
            j += 1
        g = j - i
        take = min(left, float(g))
        f[i:j] = take / g
        left -= take
        i = j
    out = torch.zeros_like(f)
    out[order] = f
    return out


def atomic_density(symbol, Z, basis, device="cuda", iters=40, damping=0.5, max_l=None):
    """Alpha density of a free atom (fractional occupation, spin averaged); max_l: the
    molecule's shell cut (Molecule.max_l)."""
    key = (symbol.upper(), basis, str(device), max_l)
    if key in _ATOM_CACHE:
        return _ATOM_CACHE[key]
    from .engine import GpuEngine
    from .molecule import N_ELECTRONS, Molecule
    ne = N_ELECTRONS[symbol.upper()]
    mol = Molecule([[symbol, Z, 0.0, 0.0, 0.0]], basis, multiplicity=1 + (ne % 2), max_l=max_l)
    eng = GpuEngine(mol, device=device).prepare()
    S, H = eng.S, eng.H
    s, U = eigen.eigh(S)
    keep = s > 1e-6
    X = (U[:, keep] * s[keep].rsqrt()).contiguous()

    from .dense import mm

    def density(F):
        e, Cp = eigen.eigh(mm(X, mm(F, X), ta=True))
        C = mm(X, Cp)
        f = _fractional_occupations(e, ne / 2.0)
        return mm(C * f, C, tb=True)

    D = density(H)
    for _ in range(iters):
        Dn = density(eng.fock(D))
        if float((Dn - D).abs().max()) < 1e-7:
            D = Dn
            break
        D = damping * D + (1.0 - damping) * Dn
    _ATOM_CACHE[key] = D
    return D


def sad_density(mol, device="cuda"):
    n = mol.NOrbitals
    D = torch.zeros(n, n, dtype=torch.float64, device=device)
    ao = 0
    first_shell = 0
    for ia, (sym, Z, _) in enumerate(mol.atoms):
        Da = atomic_density(sym, Z, mol.Basis, device, max_l=getattr(mol, "max_l", None))
        na = Da.shape[0]
        D[ao:ao + na, ao:ao + na] = Da
        ao += na
    return D
