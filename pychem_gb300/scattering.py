"""Total electron-scattering intensities on the GPU (Methods/properties.py:6-37).

For each momentum transfer S of the grid and each Hartree-Fock state,

    I(S) = N + sum_abcd [P_ab P_cd - (Pa_ad Pa_cb + Pb_ad Pb_cb)] (ab|j0(S r12)|cd),

the two-particle density of the state contracted with the scattering integrals
(``properties.py:41-73``).  Per grid value the engine switches its two-electron
operator to j0(S r12) (``pcg_scattering_class``), screens quartets with that operator's
own Schwarz bounds (``hartree_fock.py:241-327`` with ``ints_type = 1``), fills the
store, and the unrestricted digestion contracts it with every state's densities:
the sum equals sum P_a (F_a - H) + P_b (F_b - H) with the Fock matrices of that
operator.  Upstream evaluates the integrals into the tensor that still holds the
previous pass's values and skips the screened quartets, so those keep stale values;
here every grid value starts from an empty store (the intensities of a freshly zeroed
tensor).
"""
import torch

from .engine import GpuEngine


def intensities(mol, grid, densities):
    """I(S) for every grid value (rows) and state (columns) as a NumPy array.

    densities: list of (D_alpha, D_beta) per state (nbf x nbf, device or host arrays).
    An engine of its own (FP64) holds the scattering stores, one grid value at a time."""
    eng = GpuEngine(mol)
    eng.one_electron()
    dev = eng.dev
    states = [(torch.as_tensor(a, dtype=torch.float64, device=dev).contiguous(),
               torch.as_tensor(b, dtype=torch.float64, device=dev).contiguous()) for a, b in densities]
    n_el = float(mol.NElectrons)
    vals = []
    try:
        for S in grid:
            eng.scattering = float(S)
            eng.schwarz()
            eng.build_tasks()
            eng.compute_eris()
            row = []
            for Da, Db in states:
                Fa, Fb = eng.fock_u(Da, Db)
                row.append((Da * (Fa - eng.H)).sum() + (Db * (Fb - eng.H)).sum())
            vals.append(torch.stack(row))
    finally:
        eng.scattering = None
    return n_el + torch.stack(vals).cpu().numpy()


def state_densities(result):
    """(D_alpha, D_beta) of an SCF result (an RHF result's D is the density of each
    spin)."""
    if "Da" in result:
        return result["Da"], result["Db"]
    return result["D"], result["D"]
