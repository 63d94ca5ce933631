"""Non-orthogonal configuration interaction over Hartree-Fock determinants, on the GPU.

The reference's NOCI (``Methods/noci.py``) runs after the Hartree-Fock states that
``Util/structures.py:526-620`` (set_excitations) lists.  This module builds those states
(excited_states), runs their SCFs in the reference's order with its starting orbitals
(hf_states, ``pychem.py:62-93``), rearranges orbitals into spin-flip determinants
(determinants, ``noci.py:127-173``) and evaluates the CI matrix (noci_matrix,
``noci.py:51-109``):

* Lowdin pairing of each pair's occupied orbitals by a batched SVD of C1_o^T S C2_o, the
  second orbital of a pair sign-flipped when its plain dot product with the first is
  negative (``noci.py:183-205``); where upstream leaves the pairing to the solver
  (degenerate singular values) or the phase to rounding (a vanishing dot product),
  canonical choices make the CI matrix a continuous function of the orbitals
  (_canonical, _pair);
* paired overlaps, the reduced overlap over those above 1e-8 and the zero list
  (``noci.py:215-223``); co-densities W = sum_i c1_i c2_i^T / s_i, or the pair densities
  P of a zero (``noci.py:207-213,261-300``);
* J[W] and K[W] of every co-density from the ERI store by the unrestricted digestion
  kernel (GpuEngine.coulomb_exchange), the matrix elements of the no-, one- and
  two-zero forms (``noci.py:243-300``; the two-zero form takes the first zero's index in
  both spins, as upstream), 0 for more zeros, times the reduced overlap plus E_nuc
  times the determinant overlap;
* the generalised eigenproblem H v = E S v by a Cholesky factor of S and the FP64
  eigensolver (``noci.py:109``, scipy.linalg.eigh upstream).
"""
import torch

from . import eigen
from .molecule import N_ELECTRONS
from .scf import uhf

NOCI_THRESH = 1.0e-8          # Data/constants.py:37

CORE_ORBITALS = ((2, 0), (10, 1), (18, 5), (36, 9))   # Data/constants.py:10-13 by nuclear charge


def n_core_orbitals(charges):
    """Frozen-core orbital count of a molecule (Data/constants.py:10-13)."""
    total = 0
    for z in charges:
        for zmax, nc in CORE_ORBITALS:
            if z <= zmax:
                total += nc
                break
        else:
            raise ValueError("no core-orbital count for Z = %d" % z)
    return total


# ------------------------------------------------------------------------------------
# State lists (Util/structures.py:526-763)
# ------------------------------------------------------------------------------------
def _singles(o0, o1, v0, v1):
    return [[i, a] for i in range(o0, o1) for a in range(v0, v1)]


def _doubles(o0, o1, v0, v1):
    return [[i, j, a, b] for i in range(o0, o1) for j in range(i + 1, o1)
            for a in range(v0, v1) for b in range(a + 1, v1)]


def _excite(ground, ex):
    occ = list(ground)
    occ[ex[0]], occ[ex[1]] = 0, 1
    return occ


def _excite2(ground, ex):
    occ = list(ground)
    occ[ex[0]] = occ[ex[1]] = 0
    occ[ex[2]] = occ[ex[3]] = 1
    return occ


def _spinflip_states(alpha, beta, na, nb, level, istate):
    """Util/structures.py:721-746.  Mutates ``beta`` and stores the two lists
    themselves in its first entry, as upstream does: a later call that changes them
    changes that entry too."""
    beta[nb - 1] = 0
    beta[na] = 1
    out = []
    if level == 1:
        out.append([level, alpha, beta])
        for i in range(nb - 1, na):
            a, b = list(alpha), list(beta)
            a[i], b[i] = 0, 1
            a[na], b[na] = 1, 0
            out.append([istate, a, b])
    if level == 2:
        beta[nb - 2] = 0
        beta[na + 1] = 1
        out.append([level, alpha, beta])
        for i in range(nb - 2, na):
            for k in range(na, na + 2):
                a, b = list(alpha), list(beta)
                a[i], b[i] = 0, 1
                a[k], b[k] = 1, 0
                out.append([level, a, b])
            for j in range(i, na):
                a, b = list(alpha), list(beta)
                a[i] = a[j] = 0
                b[i] = b[j] = 1
                a[na] = a[na + 1] = 1
                b[na] = b[na + 1] = 0
                out.append([istate, a, b])
    return out


def _ci_states(alpha, beta, na, nb, ci_level, sf_level, istate):
    """Util/structures.py:750-798: single and double substitutions of the spin-flip
    window up to ci_level, each spin separately and combined."""
    singles = _singles(nb - sf_level, nb, na, na + sf_level)
    if sf_level == 2 and istate == 2:
        excluded = _singles(nb - 1, nb, na, na + 1)
        singles = [s for s in singles if s not in excluded]
    a1 = [_excite(alpha, s) for s in singles]
    b1 = [_excite(beta, s) for s in singles]
    a2, b2 = [], []
    if sf_level > 1:
        for d in _doubles(nb - sf_level, nb, na, na + sf_level):
            a2.append(_excite2(alpha, d))
            b2.append(_excite2(beta, d))
    out = []
    if ci_level > 0:
        out += [[istate, a, beta] for a in a1] + [[istate, alpha, b] for b in b1]
    if ci_level > 1:
        out += [[istate, a, b] for a in a1 for b in b1]
        out += [[istate, a, beta] for a in a2] + [[istate, alpha, b] for b in b2]
    if ci_level > 2:
        out += [[istate, a, b] for a in a2 for b in b1] + [[istate, a, b] for a in a1 for b in b2]
    if ci_level > 3:
        out += [[istate, a, b] for a in a2 for b in b2]
    return out


EXCITATION_ALIASES = {"CUSTOM-SINGLES": "CUSTOM-SINGLE", "DOUBLES-PAIRED": "DOUBLE-PAIRED", "SINGLE": "S",
                      "SINGLES": "S", "DOUBLE": "D", "DOUBLES": "D", "SINGLE-DOUBLE": "SD", "SINGLES-DOUBLES": "SD",
                      "SPIN-FLIP-SINGLE": "SFS", "SPIN-FLIP-SINGLES": "SFS", "SF-S": "SFS",
                      "SPIN-FLIP-DOUBLE": "SFD", "SPIN-FLIP-DOUBLES": "SFD", "SF-D": "SFD",
                      "SPIN-FLIP-SINGLE-DOUBLE": "SFSD", "SPIN-FLIP-SINGLES-DOUBLES": "SFSD", "SF-SD": "SFSD"}
EXCITATION_TYPES = {None, "HOMO-LUMO", "CUSTOM-SINGLE", "CUSTOM-PAIRED", "S", "D", "SD", "DOUBLE-PAIRED",
                    "SFS", "SFD", "SFSD", "SFS-CISD", "SFD-CISD", "SFD-CISDT", "SFD-CISDTQ", "SFSD-CISD",
                    "SFSD-CISDT", "SFSD-CISDTQ"}


def excited_states(na, nb, norb, excitations=None, n_core=0, alpha_excitations=None, beta_excitations=None):
    """Hartree-Fock state occupancies and spin-flip determinant list of
    Util/structures.py:526-657 (set_excitations).

    Returns (states, spin_flip): states is a list of (alpha, beta) occupancy lists,
    ground state first; spin_flip a list of [state index, alpha, beta] (empty unless a
    spin-flip type).  ``excitations`` takes the upstream keywords and aliases
    (Util/structures.py:393-413).  Custom lists (alpha_excitations /
    beta_excitations, upstream's CUSTOM-SINGLE and CUSTOM-PAIRED) pass upstream's
    input check, but set_excitations has no branch for them and stops
    (structures.py:614-618); they raise ValueError here."""
    exc = excitations.upper() if isinstance(excitations, str) else excitations
    exc = EXCITATION_ALIASES.get(exc, exc)
    if exc is None and (alpha_excitations or beta_excitations):
        exc = "CUSTOM-PAIRED" if (alpha_excitations and beta_excitations) else "CUSTOM-SINGLE"
    if exc not in EXCITATION_TYPES:
        raise ValueError("excitation type %r not recognised" % (excitations,))
    if exc is not None and exc.startswith("CUSTOM"):
        raise ValueError("excitation type %s not recognised in set_excitations" % exc)
    alpha_g = [1] * na + [0] * (norb - na)
    beta_g = [1] * nb + [0] * (norb - nb)
    states = [(list(alpha_g), list(beta_g))]
    if exc is None:
        return states, []
    spin_flip = []
    a_ex = b_ex = a_dbl = b_dbl = []
    if exc == "DOUBLE-PAIRED":
        a_ex = _singles(n_core, nb, na, norb)
    elif exc == "HOMO-LUMO":
        a_ex = _singles(na - 1, na, na, na + 1)
    elif exc in ("S", "D", "SD"):
        a_ex, b_ex = _singles(n_core, na, na, norb), _singles(n_core, nb, nb, norb)
        a_dbl, b_dbl = _doubles(n_core, na, na, norb), _doubles(n_core, nb, nb, norb)
    if "SF" in exc:
        spin_flip = [[0, list(alpha_g), list(beta_g)]]
        ao, bo = list(alpha_g), list(beta_g)
        ci_level = 4 if "CISDTQ" in exc else 3 if "CISDT" in exc else 2 if "CISD" in exc else 1 if "CIS" in exc else 0
        ao[na], bo[nb - 1] = 1, 0
        if "SFS" in exc:
            states.append((list(ao), list(bo)))
            if "CI" in exc:
                spin_flip += _ci_states(alpha_g, beta_g, na, nb, min(ci_level, 2), 1, 1)
            else:
                spin_flip += _spinflip_states(alpha_g, beta_g, na, nb, 1, 1)
        if ao[-1] == 0:
            ao[na + 1], bo[nb - 2] = 1, 0
        if "SFSD" in exc:
            states.append((list(ao), list(bo)))
            if "CI" in exc:
                spin_flip += _ci_states(alpha_g, beta_g, na, nb, ci_level, 2, 2)
            else:
                spin_flip += _spinflip_states(alpha_g, beta_g, na, nb, 2, 2)
        if "SFD" in exc:
            states.append((list(ao), list(bo)))
            if "CI" in exc:
                spin_flip += _ci_states(alpha_g, beta_g, na, nb, ci_level, 2, 1)
            else:
                spin_flip += _spinflip_states(alpha_g, beta_g, na, nb, 1, 1)
                spin_flip += _spinflip_states(alpha_g, beta_g, na, nb, 2, 1)
        return states, [[s[0], list(s[1]), list(s[2])] for s in spin_flip]
    beta_o = beta_g
    for ex in a_ex:
        alpha_o = _excite(alpha_g, ex)
        if exc in ("S", "SD", "HOMO-LUMO"):
            beta_o = beta_g
        if exc == "DOUBLE-PAIRED":
            beta_o = list(alpha_o)
        states.append((list(alpha_o), list(beta_o)))
    if exc in ("S", "SD"):
        for ex in b_ex:
            states.append((list(alpha_g), _excite(beta_g, ex)))
    if exc in ("D", "SD"):
        for ea in a_ex:
            for eb in b_ex:
                states.append((_excite(alpha_g, ea), _excite(beta_g, eb)))
        for ex in a_dbl:
            states.append((_excite2(alpha_g, ex), list(beta_g)))
        for ex in b_dbl:
            states.append((list(alpha_g), _excite2(beta_g, ex)))
    return states, []


# ------------------------------------------------------------------------------------
# Hartree-Fock states in the reference's order (pychem.py:62-93)
# ------------------------------------------------------------------------------------
def reorder_mos(C, occupancy):
    """Util/structures.py:979-994: swap the newly occupied orbitals above the electron
    count with the newly emptied ones below it, pairwise in order."""
    n = sum(occupancy)
    frm = [i for i in range(n) if occupancy[i] == 0]
    to = [i for i in range(n, C.shape[1]) if occupancy[i] == 1]
    C = C.clone()
    for f, t in zip(frm, to):
        C[:, [f, t]] = C[:, [t, f]]
    return C


def hf_states(engine, states, spin_flip=False, reference="UHF", constrain_excited=False, use_mom=True,
              max_iter=300, e_tol=1e-10, d_tol=1e-8):
    """SCF of every state (pychem.py:62-93, one basis set): for spin-flip lists the
    highest-spin state first, otherwise the ground state first, from the core guess;
    each later state starts from its predecessor's orbitals -- for a spin-flip state
    with unequal spin occupancies both spins from the predecessor's alpha orbitals (with
    the beta HOMO-region swaps of pychem.py:82-88 for unconstrained UHF), otherwise
    reorder_mos of the predecessor's orbitals -- and, with use_mom, keeps them occupied
    by maximum overlap (FIXED reference).  CUHF applies to every state for a CUHF
    reference, and to the excited ones with constrain_excited (hartree_fock.py:99).
    Returns one SCFResult per state, in state order."""
    if reference not in ("UHF", "CUHF"):
        raise ValueError("excited and spin-flip states need a UHF or CUHF reference")
    mol = engine.mol
    order = list(range(len(states)))
    if spin_flip:
        order.reverse()
    out = [None] * len(states)

    def run(idx, C0):
        oa, ob = states[idx]
        tot = [a + b for a, b in zip(oa, ob)]
        constrained = reference == "CUHF" or (constrain_excited and idx != 0)
        return uhf(engine, cuhf=constrained, max_iter=max_iter, e_tol=e_tol, d_tol=d_tol, C0=C0,
                   mom=use_mom and C0 is not None, occ=(sum(oa), sum(ob)),
                   cuhf_spaces=(tot.count(2), tot.count(1)))

    out[order[0]] = run(order[0], None)
    for k in range(1, len(order)):
        idx, prev = order[k], order[k - 1]
        oa, ob = states[idx]
        pa, _ = states[prev]
        C0 = None
        if spin_flip and oa != ob:
            Ca, Cb = out[prev].Ca.clone(), out[prev].Ca.clone()
            keep = constrain_excited and idx != 0
            if reference == "UHF" and not keep:
                for s in range(sum(pa) - sum(oa)):
                    t, f = sum(ob) - 1 + s, sum(pa) - 1 - s
                    Cb[:, [f, t]] = Cb[:, [t, f]]
            C0 = (Ca, Cb)
        elif mol.NAlphaElectrons == sum(oa):
            C0 = (reorder_mos(out[prev].Ca, oa), reorder_mos(out[prev].Cb, ob))
        out[idx] = run(idx, C0)
    return out


def assemble(occupancy, C, hf_occupancy):
    """Methods/noci.py:127-146: occupied columns of ``C`` (each must be occupied in its
    Hartree-Fock state) first in order, the unoccupied ones after them."""
    n = sum(occupancy)
    cols = [None] * len(occupancy)
    k_occ, k_virt = 0, n
    for i, o in enumerate(occupancy):
        if o == 0:
            cols[k_virt] = i
            k_virt += 1
        elif o == 1 and hf_occupancy[i] == 1:
            cols[k_occ] = i
            k_occ += 1
        else:
            raise ValueError("spin-flip determinant needs an orbital its Hartree-Fock state leaves empty")
    return C[:, cols]


def determinants(states, results, spin_flip_list):
    """NOCI determinants (alpha and beta orbitals): the Hartree-Fock states themselves,
    or for spin-flip lists each entry's occupancies applied to the alpha orbitals of
    its Hartree-Fock state for both spins (Methods/noci.py:149-173)."""
    if not spin_flip_list:
        return [r.Ca for r in results], [r.Cb for r in results]
    da, db = [], []
    for idx, oa, ob in spin_flip_list:
        C, hf_occ = results[idx].Ca, states[idx][0]
        da.append(assemble(oa, C, hf_occ))
        db.append(assemble(ob, C, hf_occ))
    return da, db


# ------------------------------------------------------------------------------------
# CI matrix (Methods/noci.py:51-109)
# ------------------------------------------------------------------------------------
DEGENERATE = 1.0e-8           # singular values closer than this form one cluster


def _canonical(U, V, s):
    """Fix the singular vectors inside each cluster of equal singular values.

    An SVD determines them only up to a rotation inside such a cluster (and, for the
    zero cluster, independent rotations of U and V), while upstream's two-zero element
    (noci.py:279-300) reads single pairs out of it, so its value follows the solver's
    arbitrary choice and jumps under rounding-level changes of the orbitals.  Here each
    cluster's columns become the eigenvectors of U_c^T diag(1..n) U_c (V_c^T diag(1..n)
    V_c for the zero cluster's V), ordered by eigenvalue: a choice that depends only on
    the subspaces and varies continuously with them.  Elements that do not depend on
    the basis (all others) are unchanged; signs are left to the phase rule."""
    P, n = s.shape
    if n < 2:
        return U, V
    dev, dt = s.device, s.dtype
    zero = s <= NOCI_THRESH
    split = ((s[:, :-1] - s[:, 1:]) > DEGENERATE) | (zero[:, :-1] != zero[:, 1:])
    brk = torch.cat([torch.ones(P, 1, dtype=torch.bool, device=dev), split & ~(zero[:, :-1] & zero[:, 1:])], dim=1)
    label = torch.cumsum(brk.to(torch.int64), dim=1)                      # 1, 2, ... per cluster
    same = label.unsqueeze(2) == label.unsqueeze(1)
    Dg = torch.arange(1, n + 1, dtype=dt, device=dev)
    shift = torch.diag_embed(label.to(dt) * (4.0 * n))                    # keeps blocks apart

    def rotation(X, blocks):
        K = (X.transpose(1, 2) * Dg) @ X
        K = 0.5 * (K + K.transpose(1, 2))
        _, Q = torch.linalg.eigh(torch.where(blocks, K, torch.zeros((), dtype=dt, device=dev)) + shift)
        return Q

    Qu = rotation(U, same)
    # V follows U's rotation except in the zero cluster, whose V columns get their own
    # (both matrices are block diagonal over the same clusters)
    Qv = torch.where(zero.unsqueeze(1), rotation(V, same), Qu)
    return U @ Qu, V @ Qv


def _first_large_sign(X):
    """Per column: the sign of its first entry with at least half the largest
    magnitude (a sign choice that small changes of X do not flip)."""
    mag = X.abs()
    big = mag >= 0.5 * mag.amax(dim=1, keepdim=True)
    k = big.to(torch.int8).argmax(dim=1, keepdim=True)
    return torch.where(X.gather(1, k) < 0, -1.0, 1.0).to(X.dtype)


def _pair(C1, C2, S, n):
    """Batched Lowdin pairing (noci.py:183-205): C1, C2 (P, nbf, >= n); singular
    vectors canonical inside degenerate clusters (_canonical).

    Phases as upstream: the second orbital of a pair flips when the plain dot product
    of the two is negative.  Where that dot product vanishes (orbitals of different
    symmetry on disjoint functions) upstream's choice is rounding noise; there the pair
    keeps a positive overlap if it has one, and a zero-overlap pair fixes each orbital's
    sign by its first large coefficient."""
    A, B = C1[:, :, :n], C2[:, :, :n]
    U, s, Vh = torch.linalg.svd(A.transpose(1, 2) @ S @ B)
    U, V = _canonical(U, Vh.transpose(1, 2), s)
    A2, B2 = A @ U, B @ V
    dot = (A2 * B2).sum(dim=1)
    ov = ((A2.transpose(1, 2) @ S) * B2.transpose(1, 2)).sum(dim=2)
    tiny = dot.abs() <= 1e-10 * A2.norm(dim=1) * B2.norm(dim=1)
    zero = tiny & (ov.abs() <= NOCI_THRESH)
    A2 = torch.where(zero.unsqueeze(1), A2 * _first_large_sign(A2), A2)
    B2 = torch.where(zero.unsqueeze(1), B2 * _first_large_sign(B2), B2)
    flip = torch.where(tiny, ~zero & (ov < 0), dot < 0)
    return A2, torch.where(flip.unsqueeze(1), -B2, B2)


def noci_matrix(engine, dets_a, dets_b, na, nb, return_pairs=False, max_pairs=None):
    """CI Hamiltonian and overlap over the determinants (lower triangle with the
    row's determinant as the bra, mirrored), as Methods/noci.py:55-106, without a
    host round trip: zero-overlap cases are masks, the first zero's orbital pair a
    column gather, and the J/K of all pairs' co-densities one batched digestion.
    Pairs are evaluated in chunks of at most max_pairs (default: about 2 GB of
    per-pair matrices).  With return_pairs, also the lower-triangle indices and the
    paired orbitals (a1, a2, b1, b2), one row per pair."""
    S = engine.S
    e_nuc = engine.mol.nuclear_repulsion()
    m = len(dets_a)
    dev = S.device
    f64 = torch.float64
    nbf = S.shape[0]
    ii, jj = torch.tril_indices(m, m, device=dev).unbind(0)
    Da, Db = torch.stack(dets_a), torch.stack(dets_b)
    P = ii.numel()
    if max_pairs is None:
        max_pairs = max(1, int(2.0e9 // (96 * nbf * nbf)))
    parts = [_pair_elements(engine, Da, Db, ii[k:k + max_pairs], jj[k:k + max_pairs], na, nb, e_nuc)
             for k in range(0, P, max_pairs)]
    hval = torch.cat([x[0] for x in parts])
    s_state = torch.cat([x[1] for x in parts])
    Hci = torch.zeros(m, m, dtype=f64, device=dev)
    Sci = torch.zeros_like(Hci)
    Hci[ii, jj] = hval
    Hci[jj, ii] = hval
    Sci[ii, jj] = s_state
    Sci[jj, ii] = s_state
    if return_pairs:
        return Hci, Sci, (ii, jj) + tuple(torch.cat([x[k] for x in parts]) for k in range(2, 6))
    return Hci, Sci


def _pair_elements(engine, Da, Db, ii, jj, na, nb, e_nuc):
    """Elements and overlaps of the pairs (ii[p], jj[p]) (noci.py:63-106); returns
    (H values, overlaps, a1, a2, b1, b2)."""
    S, H = engine.S, engine.H
    dev = S.device
    f64 = torch.float64
    P, nbf = ii.numel(), S.shape[0]
    empty = torch.zeros(P, nbf, 0, dtype=f64, device=dev)
    a1, a2 = _pair(Da[ii], Da[jj], S, na) if na else (empty, empty)
    b1, b2 = _pair(Db[ii], Db[jj], S, nb) if nb else (empty, empty)

    def diag(x1, M, x2):                                     # diag(x1^T M x2) per pair
        return ((x1.transpose(1, 2) @ M) * x2.transpose(1, 2)).sum(dim=2)

    ov_a, ov_b = diag(a1, S, a2), diag(b1, S, b2)
    core_a, core_b = diag(a1, H, a2), diag(b1, H, b2)
    s_state = ov_a.prod(dim=1) * ov_b.prod(dim=1)
    keep_a, keep_b = ov_a > NOCI_THRESH, ov_b > NOCI_THRESH
    inv_a = torch.where(keep_a, 1.0 / torch.where(keep_a, ov_a, 1.0), 0.0)
    inv_b = torch.where(keep_b, 1.0 / torch.where(keep_b, ov_b, 1.0), 0.0)
    reduced = torch.where(keep_a, ov_a, 1.0).prod(dim=1) * torch.where(keep_b, ov_b, 1.0).prod(dim=1)
    nz_a, nz_b = (~keep_a).sum(dim=1), (~keep_b).sum(dim=1)
    nz = nz_a + nz_b
    # the zero list runs over alpha indices, then beta: its first entry
    first_a = torch.where(~keep_a, torch.arange(na, device=dev), na).amin(dim=1) if na else nz_a
    first_b = torch.where(~keep_b, torch.arange(nb, device=dev), nb).amin(dim=1) if nb else nz_b
    spin_a = nz_a > 0
    z = torch.where(spin_a, first_a, first_b)

    def pair_density(x1, x2, n):                             # outer(x1[:, z], x2[:, z]), 0 where z >= n
        if n == 0:
            return torch.zeros(P, nbf, nbf, dtype=f64, device=dev), torch.zeros(P, dtype=torch.bool, device=dev)
        idx = z.clamp(max=n - 1).view(P, 1, 1).expand(P, nbf, 1)
        return x1.gather(2, idx) @ x2.gather(2, idx).transpose(1, 2), z < n

    Pa, in_a = pair_density(a1, a2, na)
    Pb, in_b = pair_density(b1, b2, nb)
    one, two = nz == 1, nz == 2
    Pa = Pa * ((two & in_a) | (one & spin_a)).view(P, 1, 1)
    Pb = Pb * ((two & in_b) | (one & ~spin_a)).view(P, 1, 1)
    Wa = (a1 * inv_a.unsqueeze(1)) @ a2.transpose(1, 2)
    Wb = (b1 * inv_b.unsqueeze(1)) @ b2.transpose(1, 2)
    t2 = two.view(P, 1, 1)
    Wa, Wb = torch.where(t2, Pa, Wa), torch.where(t2, Pb, Wb)
    J, K = engine.coulomb_exchange(torch.cat([Wa, Wb]))
    Jt, Xa, Xb = J[:P] + J[P:], -K[:P], -K[P:]

    def inner(x, y):
        return (x * y).sum(dim=(1, 2))

    e0 = 0.5 * (inner(Wa + Wb, Jt) + inner(Wa, Xa) + inner(Wb, Xb))
    e0 = e0 + (core_a * inv_a).sum(dim=1) + (core_b * inv_b).sum(dim=1)
    sa = spin_a.view(P, 1, 1)
    Pact, Xact = torch.where(sa, Pa, Pb), torch.where(sa, Xa, Xb)
    e12 = inner(Pact, Jt) + inner(Pact, Xact)
    zc_a = core_a.gather(1, first_a.clamp(max=max(na - 1, 0)).view(P, 1)).squeeze(1) if na else e12 * 0
    zc_b = core_b.gather(1, first_b.clamp(max=max(nb - 1, 0)).view(P, 1)).squeeze(1) if nb else e12 * 0
    e12 = e12 + torch.where(one, torch.where(spin_a, zc_a, zc_b), 0.0)
    elem = torch.where(nz == 0, e0, torch.where(nz <= 2, e12, 0.0))
    hval = elem * reduced + e_nuc * s_state
    return hval, s_state, a1, a2, b1, b2


def generalized_eigh(Hci, Sci):
    """Solutions of H v = E S v with v^T S v = 1, ascending E: S = L L^T, the FP64
    eigensolver on L^-1 H L^-T, v = L^-T y."""
    L = torch.linalg.cholesky(Sci)
    Li = torch.linalg.solve_triangular(L, torch.eye(L.shape[0], dtype=L.dtype, device=L.device), upper=False)
    A = Li @ Hci @ Li.T
    e, Y = eigen.eigh(0.5 * (A + A.T))
    return e, Li.T @ Y


def run(engine, excitations, reference="UHF", constrain_excited=False, max_iter=300, e_tol=1e-10, d_tol=1e-8):
    """The whole NOCI calculation of Methods/noci.py:51-122 after pychem.py:62-93:
    states, their SCFs, determinants, CI matrix and energies.  Returns a dict with
    ``states`` (occupancies), ``hf`` (SCFResults), ``energies``, ``vectors``, ``H``,
    ``S``."""
    mol = engine.mol
    na, nb = mol.NAlphaElectrons, mol.NBetaElectrons
    states, sf = excited_states(na, nb, engine.nbf, excitations,
                                n_core=n_core_orbitals([N_ELECTRONS[a[0]] for a in mol.atoms]))
    spin_flip = isinstance(excitations, str) and "SF" in EXCITATION_ALIASES.get(excitations.upper(),
                                                                                excitations.upper())
    res = hf_states(engine, states, spin_flip=spin_flip, reference=reference, constrain_excited=constrain_excited,
                    max_iter=max_iter, e_tol=e_tol, d_tol=d_tol)
    dets_a, dets_b = determinants(states, res, sf if spin_flip else [])
    Hci, Sci = noci_matrix(engine, dets_a, dets_b, na, nb)
    e, v = generalized_eigh(Hci, Sci)
    return dict(states=states, spin_flip=sf, hf=res, dets_alpha=dets_a, dets_beta=dets_b, energies=e, vectors=v,
                H=Hci, S=Sci)
