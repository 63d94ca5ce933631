"""Molecule, atoms and shells in upstream AO order.

Follows ``Util/structures.py``: coordinates ``[symbol, Z, x, y, z]`` in Angstrom by
default (``structures.py:339-360``, ``toBohr`` from ``Data/constants.py:2``); atoms in
input order, shells in basis-library order (``structures.py:464-492``), spherical
functions per shell in the rows of ``Data/transform_basis.py:3-12``; electron counts
``(N +/- (mult-1))/2`` (``structures.py:484-485``).  Contraction coefficients are
scaled by ``(2a)^{(l+1.5)/2}`` (``ScaledCCs``, ``structures.py:843``) and contracted
functions are not renormalised, as upstream.
"""
import json
import math
import os

import numpy as np

TO_BOHR = 1.8897161646320724
DATA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "basis_sets.json")
N_ELECTRONS = {"H": 1, "HE": 2, "LI": 3, "BE": 4, "B": 5, "C": 6, "N": 7, "O": 8, "F": 9, "NE": 10,
               "NA": 11, "MG": 12, "AL": 13, "SI": 14, "P": 15, "S": 16, "CL": 17, "AR": 18}
MAX_L = 2

_basis_cache = None


def basis_library():
    global _basis_cache
    if _basis_cache is None:
        with open(DATA) as fh:
            _basis_cache = json.load(fh)
    return _basis_cache


_shell_cache = {}


def element_shells(basis, sym):
    """(l, exponents, contraction coefficients) of every shell of an element, from the
    basis library, shared read-only between molecules."""
    key = (basis, sym)
    if key not in _shell_cache:
        data = basis_library()[basis]
        if sym not in data:
            raise ValueError("element %s not in basis %s" % (sym, basis))
        out = []
        for fn in data[sym]:
            l = int(fn[0])
            if l > MAX_L:
                raise NotImplementedError("shells above d are not supported (l=%d)" % l)
            exps = np.array([p[0] for p in fn[1:]], dtype=np.float64)
            ccs = np.array([p[1] for p in fn[1:]], dtype=np.float64)
            exps.flags.writeable = False
            ccs.flags.writeable = False
            out.append((l, exps, ccs))
        _shell_cache[key] = out
    return _shell_cache[key]


def clean_basis_name(name):
    """Upstream remove_punctuation (Util/structures.py:975-977)."""
    return name.replace("*", "s").replace("-", "").replace("(", "").replace(")", "").replace(",", "").upper()


def pure_norm(l):
    """Normalisation of the pure-axis Cartesian component x^l (ContractionScaling)."""
    return (math.gamma(l + 0.5) * math.gamma(0.5) ** 2) ** -0.5


class Molecule:
    def __init__(self, coords, basis="STO-3G", charge=0, multiplicity=1, units="ANGSTROM", max_l=None):
        scale = TO_BOHR if units.upper() == "ANGSTROM" else 1.0
        self.Basis = clean_basis_name(basis)
        lib = basis_library()
        if self.Basis not in lib:
            raise ValueError("basis set %s not available (have %s)" % (basis, sorted(lib)))
        self.Charge = charge
        self.Multiplicity = multiplicity
        self.max_l = max_l
        self.atoms = []
        for row in coords:
            sym = str(row[0]).upper()
            self.atoms.append((sym, float(row[1]), np.array([float(v) * scale for v in row[2:5]])))
        self.NAtom = len(self.atoms)
        shells = []
        for ia, (sym, Z, xyz) in enumerate(self.atoms):
            # max_l: upstream's Max_L, the shells above it dropped (Util/structures.py:815-826)
            shells += [(l, exps, ccs, ia) for l, exps, ccs in element_shells(self.Basis, sym)
                       if max_l is None or l <= max_l]
        self.shells = shells
        self.NCgtf = len(shells)
        ao = 0
        self.sh_ao = []
        for s in shells:
            self.sh_ao.append(ao)
            ao += 2 * s[0] + 1
        self.NOrbitals = ao
        self.NElectrons = sum(N_ELECTRONS[a[0]] for a in self.atoms) - charge
        self.NAlphaElectrons = (self.NElectrons + (multiplicity - 1)) // 2
        self.NBetaElectrons = (self.NElectrons - (multiplicity - 1)) // 2
        if self.NAlphaElectrons - self.NBetaElectrons + 1 != multiplicity or \
                self.NAlphaElectrons + self.NBetaElectrons != self.NElectrons:
            raise ValueError("charge and multiplicity inconsistent with specified molecule")

    # -- flat arrays for the device ---------------------------------------------------
    def arrays(self):
        """Flat shell/primitive/atom arrays for the device (computed once)."""
        if getattr(self, "_arrays", None) is not None:
            return self._arrays
        sh = self.shells
        sh_l = np.array([s[0] for s in sh], dtype=np.int32)
        sh_nprim = np.array([len(s[1]) for s in sh], dtype=np.int32)
        sh_prim = np.concatenate([[0], np.cumsum(sh_nprim)[:-1]]).astype(np.int32)
        sh_ao = np.array(self.sh_ao, dtype=np.int32)
        sh_atom = np.array([s[3] for s in sh], dtype=np.int32)
        at_xyz = np.array([a[2] for a in self.atoms], dtype=np.float64).reshape(-1, 3)
        sh_xyz = at_xyz[sh_atom]
        pr_exp = np.concatenate([s[1] for s in sh])
        lp = np.repeat(sh_l, sh_nprim)
        norm = np.array([pure_norm(l) for l in range(MAX_L + 1)])
        pr_cc = np.concatenate([s[2] for s in sh]) * (2.0 * pr_exp) ** ((lp + 1.5) / 2.0) * norm[lp]
        at_z = np.array([a[1] for a in self.atoms], dtype=np.float64)
        self._arrays = dict(sh_l=sh_l, sh_nprim=sh_nprim, sh_prim=sh_prim, sh_ao=sh_ao, sh_atom=sh_atom,
                            sh_xyz=np.ascontiguousarray(sh_xyz), pr_exp=pr_exp, pr_cc=pr_cc,
                            at_xyz=np.ascontiguousarray(at_xyz), at_z=at_z)
        return self._arrays

    def atom_nao(self):
        """Number of AOs of each atom (an atom's AOs are contiguous)."""
        n = [0] * self.NAtom
        for l, _, _, ia in self.shells:
            n[ia] += 2 * l + 1
        return n

    def nuclear_repulsion(self):
        """Methods/integrals.py:196-207 (sum over atom pairs of Z_i Z_j / r_ij)."""
        if getattr(self, "_enuc", None) is None:
            xyz = np.array([a[2] for a in self.atoms], dtype=np.float64).reshape(-1, 3)
            z = np.array([a[1] for a in self.atoms], dtype=np.float64)
            i, j = np.tril_indices(self.NAtom, -1)
            self._enuc = float(np.sum(z[i] * z[j] / np.linalg.norm(xyz[i] - xyz[j], axis=1)))
        return self._enuc

    def coords_list(self, units="BOHR"):
        s = 1.0 if units.upper() == "BOHR" else 1.0 / TO_BOHR
        return [[a[0], a[1]] + list(a[2] * s) for a in self.atoms]
