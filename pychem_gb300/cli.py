"""Run pychem input files on the GPU path.

    python -m pychem_gb300 input.inp [more.inp ...]

The input format is the reference's (``pychem.py:134-166``, ``Util/structures.py:23-47``):
INI sections, every value a Python literal, strings case-insensitive.  Each section is
one calculation; its results go to ``<section>.out`` next to the input and to stdout.

Keys read:

* ``Method``: HF, MP2, MP2-SCS, MP2-SOS (spin-component scaling of
  ``Methods/mp2.py:97-107``), NOCI (and NOCI-P2 variants, which upstream runs as NOCI).
* ``Reference``: RHF, UHF, CUHF; ``Constrain_Excited``.  As upstream, RHF changes only
  the printout: closed-shell ground states use the restricted SCF (equal to the
  unrestricted one there), open shells, excited states and NOCI run unrestricted.
* ``Coords``, ``Coords_Units`` (ANGSTROM, BOHR), ``Charge``, ``Multiplicity``,
  ``Max_SCF_Iterations`` (a floor here: at least 128 RHF / 300 UHF iterations with a
  density criterion, where upstream defaults to 25 and carries on unconverged),
  ``Max_L`` (shells above it dropped).
* ``Basis_Sets``: each in turn, later ones seeded by orbitals fitted from the previous
  one (``pychem.py:96-117``, pychem_gb300.basis_fit); NOCI runs in the last one.
* ``Excitations``: any upstream keyword (``Util/structures.py:393-413``); HOMO-LUMO by
  MOM from the ground state (``pychem.py:64-86``), the others through the state loop of
  pychem_gb300.noci.hf_states, spin-flip lists included.
* ``SCF_Guess = "READ"`` with ``MO_Read_Basis`` / ``MO_Read_State``, and ``Dump_MOs``:
  MO text files ``<basis>_<state>.alpha_MOs`` / ``.beta_MOs`` next to the input.
* ``Job_Type = "PROPERTY"`` with ``Property_Type = "SCATTERING"`` and
  ``Property_Grid``: the total electron-scattering intensity of every state at every
  grid value (``Methods/properties.py:6-37``, pychem_gb300.scattering), after NOCI of
  its determinants as upstream.

``Cartesian_L``, ``MOM_Reference = "MUTABLE"`` and ``Use_MOM = False`` with excited
states stop the section with ValueError (not implemented).  Printing and DIIS tuning
keys only shape upstream's output and its own SCF loop, and are ignored.
"""
import ast
import configparser
import os
import sys

import numpy as np
import torch

from . import noci, scattering
from .basis_fit import fit_orbitals
from .engine import GpuEngine
from .molecule import N_ELECTRONS, Molecule, clean_basis_name
from .scf import MP2_SCALES, rhf, rmp2, uhf, ump2


def read_sections(path):
    """[(section, {key: value})] with values parsed as literals and strings upper-cased
    (Util/structures.py:32-47)."""
    cp = configparser.ConfigParser()
    cp.optionxform = str
    if not cp.read(path):
        raise FileNotFoundError(path)
    out = []
    for sec in cp.sections():
        opts = {}
        for key, raw in cp.items(sec):
            val = ast.literal_eval(raw)
            opts[key.upper()] = val.upper() if isinstance(val, str) else val
        out.append((sec, opts))
    return out


def _coords(opts):
    units = opts.get("COORDS_UNITS", "ANGSTROM")
    return [[str(a[0]).upper(), float(a[1]), float(a[2]), float(a[3]), float(a[4])] for a in opts["COORDS"]], units


def _check_options(opts):
    """Input keys of the reference that change the model in ways this build does not
    implement stop the section instead of being ignored."""
    if opts.get("CARTESIAN_L"):
        raise ValueError("Cartesian basis functions (Cartesian_L = %r) are not available in this build: every shell "
                         "is spherical" % (opts["CARTESIAN_L"],))
    if opts.get("MOM_REFERENCE") == "MUTABLE":
        raise ValueError("MOM_Reference = MUTABLE is not available in this build (FIXED is)")
    if opts.get("USE_MOM") is False and opts.get("EXCITATIONS") is not None:
        raise ValueError("Use_MOM = False with excited states is not available in this build")


def run_section(name, opts, write, workdir="."):
    """One calculation; write(line) receives the report.  Returns a dict of results.
    MO text files (Dump_MOs, SCF_Guess = READ) live in ``workdir``."""
    if not opts.get("METHOD", "HF").startswith("NOCI") and (
            len(opts.get("BASIS_SETS", ["STO-3G"])) > 1 or opts.get("SCF_GUESS") == "READ" or opts.get("DUMP_MOS")):
        return run_bootstrap(name, opts, write, workdir)
    method = opts.get("METHOD", "HF")
    ref = opts.get("REFERENCE", "RHF")
    basis = opts.get("BASIS_SETS", ["STO-3G"])[-1]
    coords, units = _coords(opts)
    _check_options(opts)
    mol = Molecule(coords, basis, charge=int(opts.get("CHARGE", 0)), multiplicity=int(opts.get("MULTIPLICITY", 1)),
                   units=units, max_l=opts.get("MAX_L"))
    max_iter = int(opts.get("MAX_SCF_ITERATIONS", 128))
    eng = _engine(mol)
    res = {"section": name, "basis": basis, "reference": ref, "nbf": mol.NOrbitals}
    write("Section %s: %s/%s %s, %d basis functions" % (name, ref, basis, method, mol.NOrbitals))
    ref = _effective_reference(mol, opts, ref, method, write)
    if method.startswith("NOCI"):
        out = noci.run(eng, opts.get("EXCITATIONS"), reference=ref,
                       constrain_excited=bool(opts.get("CONSTRAIN_EXCITED", ref == "CUHF")),
                       max_iter=max(max_iter, 300))
        res["states"] = []
        for k, st in enumerate(out["hf"]):
            write("State %d: Final HF energy: %.11f (%d iterations%s)" % (k, st.E, st.iterations,
                                                                       "" if st.converged else ", not converged"))
            res["states"].append({"label": str(k), "E_hf": st.E, "iterations": st.iterations,
                                  "converged": bool(st.converged)})
        e = out["energies"].cpu().tolist()
        res["noci_energies"] = e
        write("NOCI determinants: %d" % len(out["dets_alpha"]))
        write("NOCI energies: " + " ".join("%.11f" % x for x in e))
        na, nb = mol.NAlphaElectrons, mol.NBetaElectrons
        dens = [(a[:, :na] @ a[:, :na].T, b[:, :nb] @ b[:, :nb].T) for a, b in zip(out["dets_alpha"], out["dets_beta"])]
        _properties(mol, opts, dens, res, write)
        return res
    if ref == "RHF":
        r = rhf(eng, max_iter=max_iter)
        states = [("ground", r)]
    elif opts.get("EXCITATIONS") not in (None, "HOMO-LUMO") or (
            opts.get("EXCITATIONS") == "HOMO-LUMO" and (ref == "CUHF" or opts.get("CONSTRAIN_EXCITED"))):
        # constrained excited states need the occupancy's CUHF spaces (hf_states)
        states = _excited_states(mol, eng, opts, ref, max_iter)
    else:
        r = uhf(eng, cuhf=ref == "CUHF", max_iter=max(max_iter, 300))
        states = [("ground", r)]
        if opts.get("EXCITATIONS") == "HOMO-LUMO":
            na = mol.NAlphaElectrons
            Ca = r.Ca.clone()
            Ca[:, [na - 1, na]] = Ca[:, [na, na - 1]]      # structures.reorder_MOs for HOMO -> LUMO
            states.append(("HOMO->LUMO (MOM)", uhf(eng, cuhf=ref == "CUHF", C0=(Ca, r.Cb.clone()), mom=True,
                                                   max_iter=max(max_iter, 300), d_tol=1e-6)))
    res["states"] = []
    for label, st in states:
        entry = {"label": label, "E_hf": st.E, "iterations": st.iterations, "converged": bool(st.converged)}
        write("State %s: Final HF energy: %.11f (%d iterations%s)" % (label, st.E, st.iterations,
                                                                       "" if st.converged else ", not converged"))
        if method.startswith("MP2"):
            sc = MP2_SCALES.get(method)
            e2 = rmp2(eng, st.C, st.eps, scale=sc) if ref == "RHF" else ump2(eng, st, scale=sc)
            entry["E_mp2_corr"] = e2
            write("State %s: MP2 correlation energy: %.11f  Total MP2 energy: %.11f" % (label, e2, st.E + e2))
        res["states"].append(entry)
    _properties(mol, opts, [scattering.state_densities(st) for _, st in states], res, write)
    return res


def _effective_reference(mol, opts, ref, method, write):
    """Upstream's Reference = RHF changes only the printout (hartree_fock.py:140,150):
    every state runs through its unrestricted SCF.  The restricted SCF here serves the
    closed-shell ground state it is equal to; an open-shell molecule, excited states or
    NOCI under RHF run as UHF."""
    if ref != "RHF":
        return ref
    if (mol.NAlphaElectrons != mol.NBetaElectrons or opts.get("EXCITATIONS") is not None
            or method.startswith("NOCI")):
        write("Reference RHF: the states run through the unrestricted SCF, as upstream's do")
        return "UHF"
    return ref


def _excited_states(mol, eng, opts, ref, max_iter):
    """Every state of an excitation keyword other than HOMO-LUMO (Util/structures.py:
    526-657) by the state loop of pychem.py:62-93 (noci.hf_states): for spin-flip lists
    the high-spin states first, each later state from its predecessor's orbitals and
    held by MOM.  Labels give each state's occupied orbitals (alpha / beta)."""
    exc = opts["EXCITATIONS"]
    lists, _ = noci.excited_states(mol.NAlphaElectrons, mol.NBetaElectrons, mol.NOrbitals, exc,
                                   n_core=noci.n_core_orbitals([N_ELECTRONS[a[0]] for a in mol.atoms]))
    spin_flip = "SF" in noci.EXCITATION_ALIASES.get(exc, exc)
    res = noci.hf_states(eng, lists, spin_flip=spin_flip, reference=ref,
                         constrain_excited=bool(opts.get("CONSTRAIN_EXCITED", ref == "CUHF")),
                         max_iter=max(max_iter, 300))

    def occupied(o):
        return ",".join(str(i) for i, x in enumerate(o) if x)

    return [("%d [%s / %s]" % (k, occupied(a), occupied(b)), r) for k, ((a, b), r) in enumerate(zip(lists, res))]


def _properties(mol, opts, densities, res, write):
    """Job_Type = PROPERTY (Methods/properties.py:6-37): the scattering table, grid value
    then one intensity per state, as upstream prints it."""
    if opts.get("JOB_TYPE") != "PROPERTY":
        return
    kind = opts.get("PROPERTY_TYPE")
    if kind != "SCATTERING":
        write("Property %s: not available in this build" % kind)
        return
    grid = [float(x) for x in opts["PROPERTY_GRID"]]
    table = scattering.intensities(mol, grid, densities)
    res["scattering"] = {"grid": grid, "intensities": table.tolist()}
    write("Grid value -> Scattering patterns for each electronic state")
    for S, row in zip(grid, table):
        write("%10.6f" % S + "".join("%16.12f" % v for v in row))


# ------------------------------------------------------------------------------------
# Several basis sets, MO text files (pychem.py:62-117, hartree_fock.py:35-52,152-154)
# ------------------------------------------------------------------------------------
def _engine(mol):
    return GpuEngine(mol).prepare()


_rhf, _uhf, _rmp2, _ump2 = rhf, uhf, rmp2, ump2


def mo_files(workdir, basis, state):
    """Upstream's MO file names: <basis without punctuation>_<state>.alpha_MOs / .beta_MOs
    (hartree_fock.py:152-154, structures.py:217-224)."""
    stem = os.path.join(workdir, "%s_%s" % (clean_basis_name(basis), state))
    return stem + ".alpha_MOs", stem + ".beta_MOs"


def _read_mos(files, nbf, state):
    fa, fb = files
    try:
        Ca, Cb = np.loadtxt(fa), np.loadtxt(fb)
    except OSError:
        raise FileNotFoundError("Could not read MO file for state %d (%s, %s)" % (state, fa, fb))
    if Ca.ndim != 2 or Cb.ndim != 2 or len(Ca) != nbf or len(Cb) != nbf:
        raise ValueError("Incorrect MOs supplied for state %d - check basis set and supply both alpha and beta sets"
                         % state)
    return Ca, Cb


def run_bootstrap(name, opts, write, workdir="."):
    """The state loop of pychem.py:62-117 over every listed basis set, for HF/MP2 with
    the ground state and (UHF/CUHF, Excitations = HOMO-LUMO) its alpha HOMO -> LUMO
    state.  First basis: the ground state from its own guess, or from MO files
    (SCF_Guess = READ with MO_Read_Basis / MO_Read_State, hartree_fock.py:35-52), the
    excited state from the ground state's orbitals with HOMO and LUMO swapped.  Each
    later basis: orbitals of every state fitted from the previous basis
    (pychem_gb300.basis_fit, basis_fit.py:6-21); the ground state restarts from its own
    guess, the excited state starts from its fitted orbitals.  With Excitations given,
    every state that starts from supplied orbitals keeps them occupied by MOM (upstream's
    MOM switch, structures.py:289-305).  Dump_MOs writes every state's orbitals in every
    basis (hartree_fock.py:152-154).  MP2 and properties use the last basis."""
    _check_options(opts)
    method = opts.get("METHOD", "HF")
    ref = opts.get("REFERENCE", "RHF")
    bases = opts.get("BASIS_SETS", ["STO-3G"])
    coords, units = _coords(opts)
    charge, mult = int(opts.get("CHARGE", 0)), int(opts.get("MULTIPLICITY", 1))
    max_iter = int(opts.get("MAX_SCF_ITERATIONS", 128))
    exc = opts.get("EXCITATIONS")
    use_mom = exc is not None
    if exc not in (None, "HOMO-LUMO"):
        write("Excitations %s: with several basis sets or MO files only HOMO-LUMO is available in this build"
              % exc)
    nstates = 2 if exc == "HOMO-LUMO" else 1
    read = None
    if opts.get("SCF_GUESS") == "READ":
        st, rb = opts.get("MO_READ_STATE"), opts.get("MO_READ_BASIS")
        if st is None or rb is None:
            raise ValueError("Must give details of files to read alpha and beta MOs from, using keywords "
                             "MO_Read_Basis and MO_Read_State")
        read = [mo_files(workdir, rb, str(x)) for x in (st if isinstance(st, list) else [st])]
    constrain_excited = bool(opts.get("CONSTRAIN_EXCITED", ref == "CUHF"))
    res = {"section": name, "reference": ref, "bases": list(bases), "per_basis": []}
    fitted = None
    for ib, basis in enumerate(bases):
        mol = Molecule(coords, basis, charge=charge, multiplicity=mult, units=units, max_l=opts.get("MAX_L"))
        eng = _engine(mol)
        dev = eng.S.device
        na, nb = mol.NAlphaElectrons, mol.NBetaElectrons
        write("Section %s: %s/%s %s, %d basis functions" % (name, ref, basis, method, mol.NOrbitals))
        ref = _effective_reference(mol, opts, ref, method, write)
        states = []
        for k in range(nstates):
            C0 = None
            if ib == 0 and read is not None:
                if k >= len(read):
                    raise IndexError("No MO file given for state %d" % k)
                C0 = _read_mos(read[k], mol.NOrbitals, k)
            elif k > 0 and ib > 0:
                C0 = fitted[k]
            elif k > 0:
                g = states[0]
                Ca = g.Ca.clone()
                Ca[:, [na - 1, na]] = Ca[:, [na, na - 1]]      # structures.reorder_MOs for HOMO -> LUMO
                C0 = (Ca, g.Cb.clone())
            if C0 is not None:
                C0 = tuple(torch.as_tensor(np.asarray(c) if not torch.is_tensor(c) else c, dtype=torch.float64,
                                           device=dev) for c in C0)
            mom = use_mom and C0 is not None
            if ref == "RHF":
                D0 = None if C0 is None else C0[0][:, :na] @ C0[0][:, :na].T
                r = _rhf(eng, max_iter=max_iter, D0=D0)
            else:
                # CUHF spaces from the state's occupancy (hartree_fock.py:361-365): the
                # HOMO -> LUMO state has two singly occupied positions
                n = mol.NOrbitals
                occ_a = [1] * na + [0] * (n - na)
                if k > 0:
                    occ_a[na - 1], occ_a[na] = 0, 1
                tot = [a + (1 if i < nb else 0) for i, a in enumerate(occ_a)]
                r = _uhf(eng, cuhf=ref == "CUHF" or (constrain_excited and k > 0), max_iter=max(max_iter, 300),
                         C0=C0, mom=mom, d_tol=1e-6 if mom else 1e-8, cuhf_spaces=(tot.count(2), tot.count(1)))
            states.append(r)
            label = "ground" if k == 0 else "HOMO->LUMO (MOM)"
            write("State %s: Final HF energy: %.11f (%d iterations%s)" % (label, r.E, r.iterations,
                                                                           "" if r.converged else ", not converged"))
            if opts.get("DUMP_MOS"):
                Ca = r.C if ref == "RHF" else r.Ca
                Cb = r.C if ref == "RHF" else r.Cb
                fa, fb = mo_files(workdir, basis, k)
                np.savetxt(fa, Ca.detach().cpu().numpy())
                np.savetxt(fb, Cb.detach().cpu().numpy())
        res["per_basis"].append({"basis": basis, "nbf": mol.NOrbitals,
                                 "E_hf": [float(r.E) for r in states],
                                 "iterations": [int(r.iterations) for r in states]})
        if ib + 1 < len(bases):
            nxt = bases[ib + 1]
            fitted = []
            for r in states:
                Ca = (r.C if ref == "RHF" else r.Ca).detach().cpu().numpy()
                Cb = (r.C if ref == "RHF" else r.Cb).detach().cpu().numpy()
                fitted.append((fit_orbitals(mol, Ca, nxt), fit_orbitals(mol, Cb, nxt)))
    res["basis"], res["nbf"] = bases[-1], mol.NOrbitals
    res["states"] = []
    for k, r in enumerate(states):
        entry = {"label": "ground" if k == 0 else "HOMO->LUMO (MOM)", "E_hf": float(r.E),
                 "iterations": int(r.iterations), "converged": bool(r.converged)}
        if method.startswith("MP2"):
            sc = MP2_SCALES.get(method)
            e2 = _rmp2(eng, r.C, r.eps, scale=sc) if ref == "RHF" else _ump2(eng, r, scale=sc)
            entry["E_mp2_corr"] = e2
            write("State %s: MP2 correlation energy: %.11f  Total MP2 energy: %.11f" % (entry["label"], e2,
                                                                                       r.E + e2))
        res["states"].append(entry)
    _properties(mol, opts, [scattering.state_densities(r) for r in states], res, write)
    return res


def run_file(path, stream=sys.stdout):
    results = []
    workdir = os.path.dirname(os.path.abspath(path))
    for name, opts in read_sections(path):
        out_path = os.path.join(workdir, name + ".out")
        with open(out_path, "w") as fh:
            def write(line):
                fh.write(line + "\n")
                stream.write(line + "\n")
            results.append(run_section(name, opts, write, workdir))
    return results


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    if not argv:
        print(__doc__.strip().splitlines()[2].strip())
        return 2
    if not torch.cuda.is_available():
        print("pychem_gb300 needs a CUDA device")
        return 1
    for path in argv:
        run_file(path)
    return 0
