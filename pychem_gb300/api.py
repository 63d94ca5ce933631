"""Public entry point: RHF (+MP2) of one molecule from host-side coordinates.

``rhf_mp2(coords, basis)`` is the call a user of this package makes: it takes the
upstream input conventions (``[[symbol, Z, x, y, z], ...]``, Angstrom by default,
``Util/structures.py:339-360``), runs every integral, the SCF and MP2 on the GPU, and
returns host-side results (energies, orbital energies, MO coefficients).
"""
import torch

from .engine import GpuEngine
from .molecule import Molecule
from .scf import rhf, rmp2


def rhf_mp2(coords, basis="6-31G", charge=0, multiplicity=1, units="ANGSTROM", precision="fp64",
            fp32_below=1e-4, mp2=True, device="cuda", e_tol=1e-10, d_tol=1e-8):
    mol = Molecule(coords, basis, charge=charge, multiplicity=multiplicity, units=units)
    eng = GpuEngine(mol, device=device, precision=precision, fp32_below=fp32_below).prepare()
    # MP2's pair tensor needs only the ERI store: it is built beside the SCF
    pre = eng.prefetch_mp2_tensor() if mp2 else None
    res = rhf(eng, e_tol=e_tol, d_tol=d_tol)
    out = dict(E_rhf=res.E, E_nuc=res.E_nuc, iterations=res.iterations, converged=res.converged,
               nbf=mol.NOrbitals, quartets=eng.stats["quartets"])
    if mp2:
        eri, ready = pre
        torch.cuda.current_stream().wait_event(ready)
        e2 = rmp2(eng, res.C, res.eps, eri=eri)
        del eri
        out["E_mp2_corr"] = e2
        out["E_mp2_total"] = res.E + e2
    out["mo_energies"] = res.eps.cpu().numpy()
    out["mo_coefficients"] = res.C.cpu().numpy()
    out["h2d_bytes"] = sum(t.numel() * t.element_size() for t in eng.d.values())
    out["d2h_bytes"] = out["mo_energies"].nbytes + out["mo_coefficients"].nbytes + 8 * 4
    return out
