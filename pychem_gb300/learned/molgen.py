"""Seeded random molecules for the learned initial guess.

Saturated acyclic molecules with 1..6 heavy atoms drawn from {C, N, O} plus hydrogens:
a random tree of heavy atoms obeying valences (C 4, N 3, O 2), hydrogens on the free
valences.  Geometry: standard single-bond lengths, tetrahedral bond directions with
random torsions, rejected on clashes, then every atom perturbed by N(0, 0.1 A).  No
molecule dataset is involved.
"""
import math

import numpy as np

VALENCE = {"C": 4, "N": 3, "O": 2}
Z = {"H": 1.0, "C": 6.0, "N": 7.0, "O": 8.0}
BOND = {("C", "C"): 1.54, ("C", "N"): 1.47, ("C", "O"): 1.43, ("N", "N"): 1.45, ("N", "O"): 1.40,
        ("O", "O"): 1.48, ("C", "H"): 1.09, ("N", "H"): 1.01, ("O", "H"): 0.96}
TET = math.acos(-1.0 / 3.0)


def bond_length(a, b):
    return BOND.get((a, b)) or BOND[(b, a)]


def _unit(v):
    return v / np.linalg.norm(v)


def _perp(u, rng):
    t = rng.normal(size=3)
    t -= np.dot(t, u) * u
    return _unit(t)


def _next_direction(dirs, rng):
    """A tetrahedral direction given the existing bond directions of an atom."""
    if len(dirs) == 0:
        return _unit(rng.normal(size=3))
    if len(dirs) == 1:
        u = dirs[0]
        p = _perp(u, rng)
        return math.cos(TET) * u + math.sin(TET) * p
    if len(dirs) == 2:
        u1, u2 = dirs
        d = _unit(-(u1 + u2))
        n = _unit(np.cross(u1, u2))
        a = TET / 2.0
        s = 1.0 if rng.random() < 0.5 else -1.0
        return _unit(math.cos(a) * d + s * math.sin(a) * n)
    return _unit(-(dirs[0] + dirs[1] + dirs[2]))


def random_molecule(rng, max_heavy=6, jitter=0.1, tries=50):
    for _ in range(tries):
        nh = int(rng.integers(1, max_heavy + 1))
        elem = [str(x) for x in rng.choice(["C", "C", "C", "N", "O"], size=nh)]
        parent = [-1]
        free = [VALENCE[elem[0]]]
        ok = True
        for k in range(1, nh):
            cand = [i for i in range(k) if free[i] > 0]
            if not cand or VALENCE[elem[k]] < 1:
                ok = False
                break
            p = int(rng.choice(cand))
            parent.append(p)
            free[p] -= 1
            free.append(VALENCE[elem[k]] - 1)
        if not ok:
            continue
        pos = [np.zeros(3)]
        dirs = [[] for _ in range(nh)]
        for k in range(1, nh):
            p = parent[k]
            d = _next_direction(dirs[p], rng)
            pos.append(pos[p] + bond_length(elem[p], elem[k]) * d)
            dirs[p].append(d)
            dirs[k].append(-d)
        atoms = [(elem[k], pos[k]) for k in range(nh)]
        for k in range(nh):
            for _h in range(free[k]):
                d = _next_direction(dirs[k], rng)
                dirs[k].append(d)
                atoms.append(("H", pos[k] + bond_length(elem[k], "H") * d))
        xyz = np.array([a[1] for a in atoms])
        dd = np.linalg.norm(xyz[:, None] - xyz[None], axis=-1) + np.eye(len(atoms)) * 10.0
        if dd.min() < 0.8:
            continue
        xyz = xyz + rng.normal(scale=jitter, size=xyz.shape)
        dd = np.linalg.norm(xyz[:, None] - xyz[None], axis=-1) + np.eye(len(atoms)) * 10.0
        if dd.min() < 0.6:
            continue
        return [[a[0], Z[a[0]]] + list(map(float, p)) for a, p in zip(atoms, xyz)]
    raise RuntimeError("could not build a molecule")


def molecules(n, seed, max_heavy=6, jitter=0.1):
    rng = np.random.default_rng(seed)
    return [random_molecule(rng, max_heavy, jitter) for _ in range(n)]
