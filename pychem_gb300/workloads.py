"""Seeded synthetic molecules for the benchmark configurations.

No molecule dataset is involved: every geometry is generated here from bond lengths
and angles, then perturbed with seeded Gaussian noise (numpy ``default_rng``).

* water(): O at the origin, O-H 0.9572 A, H-O-H 104.52 deg in the xy-plane.
* water_cluster(): 16 waters on a 4 x 2 x 2 grid with 2.9 A spacing, each rotated by a
  uniform random rotation (unit quaternion from N(0,1)^4) and jittered per atom with
  N(0, 0.05 A).  208 AO in 6-31G.
* alkane(): all-trans C_nH_{2n+2}, C-C 1.54 A, C-H 1.09 A, tetrahedral angles, jitter
  N(0, 0.03 A).  n = 12 gives 298 spherical AO in cc-pVDZ.
* ensemble(): cycles H2O, NH3, CH4, HF, CH3OH, C2H6 at equilibrium-like geometries with
  per-atom N(0, 0.08 A) perturbations.
"""
import math

import numpy as np

TET = math.degrees(math.acos(-1.0 / 3.0))  # 109.47 deg


def _rot(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def water(r=0.9572, angle=104.52):
    th = math.radians(angle)
    return [["O", 8.0, 0.0, 0.0, 0.0], ["H", 1.0, r, 0.0, 0.0],
            ["H", 1.0, r * math.cos(th), r * math.sin(th), 0.0]]


def water_cluster(nx=4, ny=2, nz=2, spacing=2.9, jitter=0.05, seed=2026):
    rng = np.random.default_rng(seed)
    base = np.array([a[2:] for a in water()], dtype=float)
    labels = [("O", 8.0), ("H", 1.0), ("H", 1.0)]
    atoms = []
    for i in range(nx):
        for j in range(ny):
            for k in range(nz):
                R = _rot(rng)
                xyz = base @ R.T + spacing * np.array([i, j, k], dtype=float)
                xyz = xyz + rng.normal(scale=jitter, size=xyz.shape)
                for (lab, Z), p in zip(labels, xyz):
                    atoms.append([lab, Z, float(p[0]), float(p[1]), float(p[2])])
    return atoms


def alkane(n=12, cc=1.54, ch=1.09, jitter=0.03, seed=2026):
    rng = np.random.default_rng(seed)
    half = math.radians(TET) / 2.0
    C = np.array([[k * cc * math.sin(half), (k % 2) * cc * math.cos(half), 0.0] for k in range(n)])
    atoms = [["C", 6.0] + list(c) for c in C]
    Hs = []
    ca = math.radians(TET) / 2.0
    for k in range(n):
        nb = [C[j] - C[k] for j in (k - 1, k + 1) if 0 <= j < n]
        u = [v / np.linalg.norm(v) for v in nb]
        if len(u) == 2:
            d = -(u[0] + u[1]); d /= np.linalg.norm(d)
            nrm = np.cross(u[0], u[1]); nrm /= np.linalg.norm(nrm)
            for s in (1, -1):
                Hs.append(C[k] + ch * (math.cos(ca) * d + s * math.sin(ca) * nrm))
        else:
            a = u[0]
            # e1 in the backbone plane, perpendicular to the C-C bond, pointing away
            # from the zigzag (anti arrangement), e2 the plane normal
            inplane = np.array([0.0, 1.0 if k % 2 == 0 else -1.0, 0.0])
            e1 = inplane - np.dot(inplane, a) * a
            e1 /= np.linalg.norm(e1)
            e1 = -e1
            e2 = np.cross(a, e1)
            ct, st = math.cos(math.radians(TET)), math.sin(math.radians(TET))
            for phi in (0.0, 2 * math.pi / 3, 4 * math.pi / 3):
                Hs.append(C[k] + ch * (ct * a + st * (math.cos(phi) * e1 + math.sin(phi) * e2)))
    for h in Hs:
        atoms.append(["H", 1.0] + list(h))
    xyz = np.array([a[2:] for a in atoms]) + rng.normal(scale=jitter, size=(len(atoms), 3))
    return [[a[0], a[1]] + list(map(float, p)) for a, p in zip(atoms, xyz)]


def twisted_ethylene(twist=90.0, cc=1.34, ch=1.086, hch=117.0):
    """C2H4 with one CH2 group rotated by ``twist`` degrees about the C=C axis (x): at
    90 degrees the pi bond is broken and the singlet is a diradical, the textbook case
    for spin-flip NOCI."""
    half = math.radians(hch / 2.0)
    out = [["C", 6.0, 0.0, 0.0, 0.0], ["C", 6.0, cc, 0.0, 0.0]]
    for c_x, sign, rot in ((0.0, -1.0, 0.0), (cc, 1.0, math.radians(twist))):
        for s in (1.0, -1.0):
            y, z = ch * math.sin(half) * s, 0.0
            y, z = y * math.cos(rot) - z * math.sin(rot), y * math.sin(rot) + z * math.cos(rot)
            out.append(["H", 1.0, c_x + sign * ch * math.cos(half), y, z])
    return out


def _tetra_dirs():
    return np.array([[1, 1, 1], [1, -1, -1], [-1, 1, -1], [-1, -1, 1]], dtype=float) / math.sqrt(3.0)


def small_molecule(name):
    """Equilibrium-like geometries built from standard bond lengths and angles."""
    if name == "H2O":
        return water()
    if name == "HF":
        return [["F", 9.0, 0.0, 0.0, 0.0], ["H", 1.0, 0.917, 0.0, 0.0]]
    if name == "NH3":
        r, ang = 1.012, math.radians(106.7)
        # three H at equal angles around z
        cos_t = math.sqrt(max(0.0, (1 + 2 * math.cos(ang)) / 3.0))
        sin_t = math.sqrt(1 - cos_t ** 2)
        out = [["N", 7.0, 0.0, 0.0, 0.0]]
        for k in range(3):
            phi = 2 * math.pi * k / 3
            out.append(["H", 1.0, r * sin_t * math.cos(phi), r * sin_t * math.sin(phi), -r * cos_t])
        return out
    if name == "CH4":
        return [["C", 6.0, 0.0, 0.0, 0.0]] + [["H", 1.0] + list(1.087 * d) for d in _tetra_dirs()]
    if name == "C2H6":
        cc, ch = 1.535, 1.094
        out = [["C", 6.0, 0.0, 0.0, 0.0], ["C", 6.0, 0.0, 0.0, cc]]
        ct = math.cos(math.radians(TET))
        st = math.sin(math.radians(TET))
        for k in range(3):
            phi = 2 * math.pi * k / 3
            out.append(["H", 1.0, ch * st * math.cos(phi), ch * st * math.sin(phi), ch * ct])
            phi2 = phi + math.pi / 3
            out.append(["H", 1.0, ch * st * math.cos(phi2), ch * st * math.sin(phi2), cc - ch * ct])
        return out
    if name == "CH3OH":
        co, ch, oh = 1.427, 1.094, 0.956
        out = [["C", 6.0, 0.0, 0.0, 0.0], ["O", 8.0, 0.0, 0.0, co]]
        ct = math.cos(math.radians(TET))
        st = math.sin(math.radians(TET))
        for k in range(3):
            phi = 2 * math.pi * k / 3 + math.pi / 3
            out.append(["H", 1.0, ch * st * math.cos(phi), ch * st * math.sin(phi), ch * ct])
        a = math.radians(108.5)
        out.append(["H", 1.0, oh * math.sin(a), 0.0, co - oh * math.cos(a)])
        return out
    raise ValueError(name)


ENSEMBLE_NAMES = ["H2O", "NH3", "CH4", "HF", "CH3OH", "C2H6"]


def ensemble(n=1024, jitter=0.08, seed=2026, names=ENSEMBLE_NAMES):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        base = small_molecule(names[i % len(names)])
        xyz = np.array([a[2:] for a in base], dtype=float) + rng.normal(scale=jitter, size=(len(base), 3))
        out.append([[a[0], a[1]] + list(map(float, p)) for a, p in zip(base, xyz)])
    return out
