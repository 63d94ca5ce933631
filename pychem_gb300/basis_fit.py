"""Orbitals carried from one basis set to the next (upstream ``Methods/basis_fit.py``).

pychem runs a list of basis sets in turn (``pychem.py:96-117``): after the states of
one basis have converged, each state's MO coefficients are projected into the next
basis and seed that basis's SCFs (the excited states' MOM references; the ground
state restarts from its own guess).  The projection is per atom, per angular momentum
l and per magnetic component m: the old contracted radial functions of that l,
weighted by the MO coefficients, are fitted by the new ones in the least-squares sense
of one-centre radial overlaps

    <g1|g2>_l = c1 c2 (a1 a2)^(3/4 + l/2) / ((a1 + a2)^(3/2) (2 (a1 + a2))^l)

(``basis_fit.py:25-32``), i.e. new = S_new^-1 T.  The index bookkeeping is upstream's
(``basis_fit.py:36-66``): within an atom the old coefficients are read as if every
l-block were contiguous and in increasing l, and the new ones are written that way,
with zeros for the new basis's polarisation shells; basis sets whose library order
interleaves l (6-31G's s, s, p, s, p for first-row atoms) therefore get their fitted
coefficients in upstream's order too.  The result is square in the new basis, fitted
columns first and zero columns for the rest (``basis_fit.py:17-21``).

This is a few hundred small dense solves on the host per state, done once per basis
change; the SCFs it seeds run on the GPU.
"""
import numpy as np

from .molecule import clean_basis_name, element_shells


def _radial_overlap(e1, c1, e2, c2, l):
    g = e1 + e2
    return c1 * c2 * (e1 * e2) ** (0.75 + 0.5 * l) / (g ** 1.5 * (2.0 * g) ** l)


def _fit_one(old_shells, coeffs, start, new_shells, l):
    """basis_fit.py:70-106: one magnetic component of one l on one atom."""
    nn = len(new_shells)
    S = np.zeros((nn, nn))
    for i, (e1, c1) in enumerate(new_shells):
        for j, (e2, c2) in enumerate(new_shells[:i + 1]):
            S[i, j] = np.sum(_radial_overlap(e1[:, None], c1[:, None], e2[None, :], c2[None, :], l))
    S += np.tril(S, -1).T
    T = np.zeros(nn)
    k = start
    for e_old, c_old in old_shells:
        w = c_old * coeffs[k]
        k += 2 * l + 1
        for i, (e1, c1) in enumerate(new_shells):
            T[i] += np.sum(_radial_overlap(e1[:, None], c1[:, None], e_old[None, :], w[None, :], l))
    return np.linalg.solve(S, T)


def fit_orbitals(mol, C, new_basis):
    """MO coefficients C (old basis of ``mol``, square) projected into ``new_basis``:
    an (n_new x n_new) array whose first n_old columns are the fitted orbitals."""
    C = np.asarray(C, dtype=np.float64)
    new_basis = clean_basis_name(new_basis)
    per_atom = []
    for ia, (sym, _, _) in enumerate(mol.atoms):
        old = [(l, e, c) for (l, e, c, a) in mol.shells if a == ia]
        per_atom.append((sym, old, element_shells(new_basis, sym)))
    cols = []
    for k in range(C.shape[0]):
        mo = C[:, k]
        new_mo = []
        start = 0
        for sym, old, new in per_atom:
            # the offset inside an atom is local (basis_fit.py:36-66); the next atom
            # starts after this atom's old functions (basis_fit.py:12-15)
            count = start
            start += sum(2 * l + 1 for l, _, _ in old)
            atom_coeffs = []
            max_old = max(l for l, _, _ in old)
            coeffs = None
            for l in range(max_old + 1):
                degen = 2 * l + 1
                old_l = [(e, c) for ll, e, c in old if ll == l]
                new_l = [(e, c) for ll, e, c in new if ll == l]
                if old_l:
                    coeffs = [0.0] * (len(new_l) * degen)
                    for m in range(degen):
                        fitted = _fit_one(old_l, mo, count + m, new_l, l)
                        for i, v in enumerate(fitted):
                            coeffs[i * degen + m] = float(v)
                # upstream appends the current list even for an l the old basis lacks
                atom_coeffs += coeffs
                count += len(old_l) * degen
            if max(l for l, _, _ in new) > max_old:
                for l, _, _ in new:
                    if l > max_old:
                        atom_coeffs += [0.0] * (2 * l + 1)
            new_mo += atom_coeffs
        cols.append(new_mo)
    n_new = len(cols[0])
    out = np.zeros((n_new, n_new))
    out[:, :len(cols)] = np.array(cols).T
    return out
