"""Run the upstream pychem reference inside this container, for fixture generation only.

The upstream code (dlc62/pychem) is Python 2 and ships without its Boys-function
table (``Methods/c_ints/interpolation_table.c`` is a missing blob; its interface is
``Methods/c_ints/interpolation_table.h:4-14``).  This helper

1. copies the read-only reference tree into a fresh temporary directory,
2. applies mechanical Python 2 -> 3 edits (tabs -> 8 spaces, ``izip``/``xrange``/
   ``sys.maxint``, integer ``//`` where the code needs an int, package ``__init__``
   files that only set up import paths),
3. writes a regenerated Boys table with the header's layout (``n_points`` = 7750,
   ``d`` = 0.0025, cubic coefficients in the absolute table coordinate
   ``sT = T/(2d)`` as consumed by ``two_electron_fundamentals.c:62-71``),
4. compiles ``_c_ints`` with gcc from the 16 sources listed in ``Methods/setup.py:5-12``,
5. imports the patched modules.

Nothing here is imported by the library, by ``smoke()`` or by ``bench.py``; the
reference tree does not exist on GPU machines.  The generated fixtures in this
folder are what travel.
"""
import math
import os
import shutil
import subprocess
import sys
import sysconfig
import tempfile

import numpy as np

REFERENCE = os.environ.get("PYCHEM_REFERENCE")  # path of the reference tree; no default

# Boys table layout fixed by interpolation_table.h:4-14
N_POINTS = 7750
D_STEP = 0.0025
M_TAB = 29


def boys_exact(mmax, T):
    """F_m(T) for m = 0..mmax at an array of T (float64), by the positive series
    F_M(T) = exp(-T) sum_k (2T)^k / ((2M+1)(2M+3)...(2M+2k+1)) for the top order and
    the stable downward recursion F_{m-1} = (2T F_m + exp(-T)) / (2m-1)."""
    T = np.asarray(T, dtype=np.float64)
    e = np.exp(-T)
    term = np.full_like(T, 1.0 / (2 * mmax + 1))
    acc = term.copy()
    k = 0
    while True:
        k += 1
        term = term * (2.0 * T) / (2 * mmax + 2 * k + 1)
        acc = acc + term
        if k > 20 and np.all(term <= 1e-18 * acc):
            break
        if k > 2000:
            raise RuntimeError("Boys series did not converge")
    out = np.empty((mmax + 1,) + T.shape)
    out[mmax] = e * acc
    for m in range(mmax, 0, -1):
        out[m - 1] = (2.0 * T * out[m] + e) / (2 * m - 1)
    return out


def write_boys_table(path):
    """Cubic per-interval Taylor expansion about each interval midpoint, re-expanded
    in the absolute coordinate sT so that f0+sT*(f1+sT*(f2+sT*f3)) reproduces F_m."""
    j = np.arange(N_POINTS, dtype=np.float64)
    s_mid = j + 0.5
    t_mid = 2.0 * D_STEP * s_mid
    F = boys_exact(M_TAB + 3, t_mid)
    h = 2.0 * D_STEP

    def coeffs(derivs):
        # derivs[k] = k-th derivative at the midpoint
        a = [derivs[k] * h ** k / math.factorial(k) for k in range(4)]
        s = s_mid
        c0 = a[0] - a[1] * s + a[2] * s * s - a[3] * s * s * s
        c1 = a[1] - 2.0 * a[2] * s + 3.0 * a[3] * s * s
        c2 = a[2] - 3.0 * a[3] * s
        c3 = a[3]
        return c0, c1, c2, c3

    f = [np.empty((M_TAB, N_POINTS)) for _ in range(4)]
    for m in range(M_TAB):
        c = coeffs([(-1) ** k * F[m + k] for k in range(4)])
        for q in range(4):
            f[q][m] = c[q]
    ex = np.exp(-t_mid)
    e = coeffs([(-1) ** k * ex for k in range(4)])

    with open(path, "w") as fh:
        fh.write('#include "interpolation_table.h"\n')
        fh.write("const int n_points = %d;\nconst double d = %.17g;\n" % (N_POINTS, D_STEP))
        for q in range(4):
            fh.write("const double e%d[%d] = {" % (q, N_POINTS))
            fh.write(",".join("%.17g" % v for v in e[q]))
            fh.write("};\n")
        for q in range(4):
            fh.write("const double f%d[%d][%d] = {" % (q, M_TAB, N_POINTS))
            rows = []
            for m in range(M_TAB):
                rows.append("{" + ",".join("%.17g" % v for v in f[q][m]) + "}")
            fh.write(",\n".join(rows))
            fh.write("};\n")


_EDITS = {
    "Data/constants.py": [("(i*i+i)/2", "(i*i+i)//2")],
    "Util/structures.py": [
        ("sys.maxint", "sys.maxsize"),
        ("(self.NElectrons + (self.Multiplicity-1))/2", "(self.NElectrons + (self.Multiplicity-1))//2"),
        ("(self.NElectrons - (self.Multiplicity-1))/2", "(self.NElectrons - (self.Multiplicity-1))//2"),
    ],
    "Methods/hartree_fock.py": [("from itertools import izip", "izip = zip"),
                                # Python 2 compared an array with [] to a scalar True;
                                # NumPy now compares elementwise
                                ("elif this_state.Alpha.MOs != []:", "elif len(this_state.Alpha.MOs) != 0:")],
    "Methods/hf_extensions/diis.py": [("xrange", "range")],
    "Methods/basis_fit.py": [("xrange", "range")],
    "pychem.py": [("SafeConfigParser", "ConfigParser")],
    # numpy.product was removed in NumPy 2
    "Methods/noci.py": [("np.product(alpha_overlaps) * np.product(beta_overlaps)",
                         "np.prod(alpha_overlaps) * np.prod(beta_overlaps)")],
}

_INITS = {
    "Data/__init__.py": "",
    "Util/__init__.py": "",
    "Methods/__init__.py": "import os, sys\nsys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))\n",
    "Methods/hf_extensions/__init__.py": "from . import diis\nfrom . import mom\n",
}

_C_SOURCES = [
    "_c_ints.c", "c_ints/shellpair_quantities.c", "c_ints/one_electron_fundamentals.c",
    "c_ints/one_electron_vrr.c", "c_ints/one_electron_hrr.c", "c_ints/one_electron_contract.c",
    "c_ints/one_electron_kinetic.c", "c_ints/two_electron_bound.c",
    "c_ints/two_electron_fundamentals.c", "c_ints/two_electron_vrr.c",
    "c_ints/two_electron_contract.c", "c_ints/two_electron_hrr.c",
    "c_ints/two_electron_scattering.c", "c_ints/spherical_bessel_j.c",
    "c_ints/angmom_index.c", "c_ints/interpolation_table.c",
]


def prepare(workdir=None):
    """Patched, built copy of the reference; returns its root directory."""
    if not REFERENCE or not os.path.isdir(REFERENCE):
        raise RuntimeError("set PYCHEM_REFERENCE to the path of the reference tree (now %r)" % REFERENCE)
    root = os.path.join(workdir or tempfile.mkdtemp(prefix="pychem_ref_"), "ref")
    shutil.copytree(REFERENCE, root, copy_function=shutil.copyfile)
    for dirpath, _, files in os.walk(root):
        for name in files:
            if name.endswith(".py"):
                p = os.path.join(dirpath, name)
                with open(p) as fh:
                    text = fh.read().expandtabs(8)
                rel = os.path.relpath(p, root)
                for old, new in _EDITS.get(rel, []):
                    if old not in text:
                        raise RuntimeError("edit anchor %r missing in %s" % (old, rel))
                    text = text.replace(old, new)
                if rel in _INITS:
                    text = _INITS[rel]
                with open(p, "w") as fh:
                    fh.write(text)
    meth = os.path.join(root, "Methods")
    write_boys_table(os.path.join(meth, "c_ints", "interpolation_table.c"))
    out = os.path.join(meth, "_c_ints" + sysconfig.get_config_var("EXT_SUFFIX"))
    cmd = ["gcc", "-O2", "-shared", "-fPIC", "-w",
           "-I" + sysconfig.get_paths()["include"], "-I" + np.get_include(),
           "-o", out] + [os.path.join(meth, s) for s in _C_SOURCES] + ["-lm"]
    subprocess.check_call(cmd)
    return root


def load(root):
    """Import the patched reference modules from ``root``; returns a namespace dict."""
    for p in (root, os.path.join(root, "Methods")):
        if p not in sys.path:
            sys.path.insert(0, p)
    import Methods  # noqa: F401  (sets up the Methods import path)
    from Data import constants
    from Util import structures
    import integrals
    import hartree_fock
    import mp2
    import _c_ints
    np.seterr(all="ignore")  # the reference's diis.py sets all='raise' at import
    constants.energy_convergence = 1e-11
    return dict(constants=constants, structures=structures, integrals=integrals,
                hartree_fock=hartree_fock, mp2=mp2, c_ints=_c_ints)


def molecule_from_spec(ns, coords, basis, charge=0, multiplicity=1, reference="RHF",
                       units="ANGSTROM", method="HF", max_iter=200, outdir=None, extra=None):
    """Build reference Settings/Molecule objects from an in-memory INI section."""
    import configparser
    cp = configparser.ConfigParser()
    cp.optionxform = str
    sec = "case"
    cp.add_section(sec)
    cp.set(sec, "Method", repr(method))
    cp.set(sec, "MP2_type", repr("AFTER"))
    cp.set(sec, "Basis_Sets", repr([basis]))
    cp.set(sec, "Multiplicity", repr(multiplicity))
    cp.set(sec, "Charge", repr(charge))
    cp.set(sec, "Coords_Units", repr(units))
    cp.set(sec, "Coords", repr([[a[0], float(a[1]), float(a[2]), float(a[3]), float(a[4])] for a in coords]))
    cp.set(sec, "Reference", repr(reference))
    cp.set(sec, "Max_SCF_Iterations", repr(max_iter))
    for key, value in (extra or {}).items():
        cp.set(sec, key, repr(value))
    molecule, settings = ns["structures"].process_input(sec, cp)
    outdir = outdir or tempfile.mkdtemp(prefix="pychem_out_")
    settings.OutFile = open(os.path.join(outdir, "case.out"), "w")
    return molecule, settings
