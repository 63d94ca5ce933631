"""Run pychem input files on the GPU path.

    python -m pychem_gb300 input.inp [more.inp ...]

The input format is the reference's (``pychem.py:134-166``, ``Util/structures.py:23-47``):
INI sections, every value a Python literal, strings case-insensitive.  Each section is
one calculation; its results go to ``<section>.out`` next to the input and to stdout.

Read keys: ``Method`` (HF, MP2), ``Reference`` (RHF, UHF, CUHF), ``Basis_Sets`` (the
calculation runs in the last one; the upstream basis-fitting bootstrap through the
earlier ones only supplies starting orbitals), ``Coords``, ``Coords_Units`` (ANGSTROM,
BOHR), ``Charge``, ``Multiplicity``, ``Max_SCF_Iterations``, ``Excitations`` (HOMO-LUMO:
the alpha HOMO -> LUMO state by MOM after the ground state, as ``pychem.py:64-86``),
``Constrain_Excited``, ``Job_Type`` / ``Property_Type`` / ``Property_Grid``.
``Method = "NOCI"`` runs the states of any ``Excitations`` keyword (spin-flip lists
included) and the NOCI of ``Methods/noci.py`` (pychem_gb300.noci).
``Job_Type = "PROPERTY"`` with ``Property_Type = "SCATTERING"`` adds the total
electron-scattering intensity of every state at every grid value
(``Methods/properties.py:6-37``, pychem_gb300.scattering), after NOCI of its
determinants as upstream.
"""
import ast
import configparser
import os
import sys

import torch

from . import noci, scattering
from .engine import GpuEngine
from .molecule import Molecule
from .scf import rhf, rmp2, uhf, ump2


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


def run_section(name, opts, write):
    """One calculation; write(line) receives the report.  Returns a dict of results."""
    method = opts.get("METHOD", "HF")
    ref = opts.get("REFERENCE", "RHF")
    basis = opts.get("BASIS_SETS", ["STO-3G"])[-1]
    coords, units = _coords(opts)
    mol = Molecule(coords, basis, charge=int(opts.get("CHARGE", 0)), multiplicity=int(opts.get("MULTIPLICITY", 1)),
                   units=units)
    max_iter = int(opts.get("MAX_SCF_ITERATIONS", 128))
    eng = GpuEngine(mol).prepare()
    res = {"section": name, "basis": basis, "reference": ref, "nbf": mol.NOrbitals}
    write("Section %s: %s/%s %s, %d basis functions" % (name, ref, basis, method, mol.NOrbitals))
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
        if mol.NAlphaElectrons != mol.NBetaElectrons:
            raise ValueError("section %s: RHF needs a closed-shell molecule" % name)
        r = rhf(eng, max_iter=max_iter)
        states = [("ground", r)]
    else:
        r = uhf(eng, cuhf=ref == "CUHF", max_iter=max(max_iter, 300))
        states = [("ground", r)]
        if opts.get("EXCITATIONS") == "HOMO-LUMO":
            na = mol.NAlphaElectrons
            Ca = r.Ca.clone()
            Ca[:, [na - 1, na]] = Ca[:, [na, na - 1]]      # structures.reorder_MOs for HOMO -> LUMO
            states.append(("HOMO->LUMO (MOM)", uhf(eng, cuhf=ref == "CUHF", C0=(Ca, r.Cb.clone()), mom=True,
                                                   max_iter=max(max_iter, 300), d_tol=1e-6)))
        elif opts.get("EXCITATIONS") is not None:
            write("Excitations %s: not available in this build" % opts["EXCITATIONS"])
    res["states"] = []
    for label, st in states:
        entry = {"label": label, "E_hf": st.E, "iterations": st.iterations, "converged": bool(st.converged)}
        write("State %s: Final HF energy: %.11f (%d iterations%s)" % (label, st.E, st.iterations,
                                                                       "" if st.converged else ", not converged"))
        if method.startswith("MP2"):
            e2 = rmp2(eng, st.C, st.eps) if ref == "RHF" else ump2(eng, st)
            entry["E_mp2_corr"] = e2
            write("State %s: MP2 correlation energy: %.11f  Total MP2 energy: %.11f" % (label, e2, st.E + e2))
        res["states"].append(entry)
    _properties(mol, opts, [scattering.state_densities(st) for _, st in states], res, write)
    return res


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


def run_file(path, stream=sys.stdout):
    results = []
    for name, opts in read_sections(path):
        out_path = os.path.join(os.path.dirname(os.path.abspath(path)), name + ".out")
        with open(out_path, "w") as fh:
            def write(line):
                fh.write(line + "\n")
                stream.write(line + "\n")
            results.append(run_section(name, opts, write))
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
