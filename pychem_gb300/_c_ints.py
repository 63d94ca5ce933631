"""Drop-in replacement for the upstream ``_c_ints`` CPython extension.

Same 11 functions, same argument order and meaning as ``Methods/_c_ints.c:68-81``:
arrays are float64 NumPy arrays, outputs are filled in place (the two ``*_contract``
functions accumulate), every function returns None.  Each call runs one kernel of
libpychem_gb300.so on the GPU (include/pychem_gb300.h, section 1).

Error behaviour: a wrong argument type raises ``TypeError("Error parsing objects
passed to C")`` as upstream; arrays too small for the requested shapes raise
ValueError (upstream reads out of bounds); output arrays must be C-contiguous and
writeable (upstream silently writes into a temporary copy otherwise).
``two_electron_fundamentals`` with ``ints_type == 1`` gives the j0(S r12) scattering
fundamentals at S = ``grid_value`` (``two_electron_scattering.c``), any other type the
1/r12 ones, as upstream branches.

Usage from the upstream tree: put this package on sys.path and ``import
pychem_gb300._c_ints as _c_ints`` in place of the compiled extension.
"""
import ctypes

import numpy as np

from . import _lib

_PARSE = "Error parsing objects passed to C"


def _nc(l):
    return 0 if l < 0 else (l + 1) * (l + 2) // 2


def _in(a, need=0):
    if isinstance(a, (list, tuple)):
        a = np.asarray(a, dtype=np.float64)
    if not isinstance(a, np.ndarray) or a.dtype != np.float64:
        raise TypeError(_PARSE)
    a = np.ascontiguousarray(a)
    if a.size < need:
        raise ValueError("array of %d elements, %d required" % (a.size, need))
    return a


def _out(a, need):
    if not isinstance(a, np.ndarray) or a.dtype != np.float64:
        raise TypeError(_PARSE)
    if not (a.flags.c_contiguous and a.flags.writeable):
        raise TypeError("output arrays must be C-contiguous and writeable")
    if a.size < need:
        raise ValueError("output array of %d elements, %d required" % (a.size, need))
    return a


def _p(a):
    if a is None or a.size == 0:
        return None
    return a.ctypes.data_as(_lib.P_DBL)


def _int(*xs):
    for x in xs:
        if not isinstance(x, (int, np.integer)) or isinstance(x, bool):
            raise TypeError(_PARSE)
    return [int(x) for x in xs]


def shellpair_quantities(sigmas, overlaps, centres, alpha_exps, A, n_alpha, beta_exps, B, n_beta):
    n_alpha, n_beta = _int(n_alpha, n_beta)
    n = n_alpha * n_beta
    s, o, c = _out(sigmas, n), _out(overlaps, n), _out(centres, 3 * n)
    ea, pa, eb, pb = _in(alpha_exps, n_alpha), _in(A, 3), _in(beta_exps, n_beta), _in(B, 3)
    _lib.call("pcg_shellpair_quantities", _p(s), _p(o), _p(c), _p(ea), _p(pa), n_alpha, _p(eb), _p(pb), n_beta)


def two_electron_bound(bounds, C_P, C_Q, nla, nlb, nlc, nld):
    nla, nlb, nlc, nld = _int(nla, nlb, nlc, nld)
    b = _out(bounds, nla * nlb * nlc * nld)
    p, q = _in(C_P, nla * nlb), _in(C_Q, nlc * nld)
    _lib.call("pcg_two_electron_bound", _p(b), _p(p), _p(q), nla, nlb, nlc, nld)


def two_electron_fundamentals(fundamentals, sigma_P, U_P, P, sigma_Q, U_Q, Q, R, na, nb, nc, nd, m, ints_type,
                              grid_value):
    na, nb, nc, nd, m, ints_type = _int(na, nb, nc, nd, m, ints_type)
    nbra, nket = na * nb, nc * nd
    f, r = _out(fundamentals, (m + 1) * nbra * nket), _out(R, 3 * nbra * nket)
    sp, up, pp = _in(sigma_P, nbra), _in(U_P, nbra), _in(P, 3 * nbra)
    sq, uq, qq = _in(sigma_Q, nket), _in(U_Q, nket), _in(Q, 3 * nket)
    _lib.call("pcg_two_electron_fundamentals", _p(f), _p(sp), _p(up), _p(pp), _p(sq), _p(uq), _p(qq), _p(r),
              na, nb, nc, nd, m, ints_type, float(grid_value))


def two_electron_vrr(target, base0, base1, base2, base3, base4, zeta, eta, kappa, Rx, R, na, nb, nc, nd, lbra, lket,
                     kappa_index):
    na, nb, nc, nd, lbra, lket, kappa_index = _int(na, nb, nc, nd, lbra, lket, kappa_index)
    npb, npk = na * nb, nc * nd
    cols = _nc(lket) * npk
    t = _out(target, _nc(lbra) * npb * cols)
    b0, b1 = _in(base0, _nc(lbra - 1) * npb * cols), _in(base1, _nc(lbra - 1) * npb * cols)
    b2 = _in(base2, _nc(lbra - 2) * npb * cols) if lbra >= 2 else None
    b3 = _in(base3, _nc(lbra - 2) * npb * cols) if lbra >= 2 else None
    b4 = _in(base4, _nc(lbra - 1) * npb * _nc(lket - 1) * npk) if lket >= 1 else None
    z, e = _in(zeta, npb), _in(eta, npk)
    k = _in(kappa, na if kappa_index == 0 else nb)
    rx, r = _in(Rx, 3), _in(R, 3 * npb * npk)
    _lib.call("pcg_two_electron_vrr", _p(t), _p(b0), _p(b1), _p(b2), _p(b3), _p(b4), _p(z), _p(e), _p(k), _p(rx),
              _p(r), na, nb, nc, nd, lbra, lket, kappa_index)


def two_electron_contract(contracted, primitive, cc_bra, cc_ket, na, nb, nc, nd, lbra, lket):
    na, nb, nc, nd, lbra, lket = _int(na, nb, nc, nd, lbra, lket)
    o = _out(contracted, _nc(lbra) * _nc(lket))
    p = _in(primitive, _nc(lbra) * na * nb * _nc(lket) * nc * nd)
    cb, ck = _in(cc_bra, na * nb), _in(cc_ket, nc * nd)
    _lib.call("pcg_two_electron_contract", _p(o), _p(p), _p(cb), _p(ck), na, nb, nc, nd, lbra, lket)


def two_electron_hrr(target, base0, base1, Rx, la, lb, lc, ld, goofy):
    la, lb, lc, ld, goofy = _int(la, lb, lc, ld, goofy)
    nket = _nc(lc) * _nc(ld)
    if goofy == 0:
        nt, n0 = _nc(la) * _nc(lb + 1), _nc(la + 1) * _nc(lb)
    else:
        nt, n0 = _nc(la + 1) * _nc(lb), _nc(la) * _nc(lb + 1)
    t = _out(target, nt * nket)
    b0, b1, rx = _in(base0, n0 * nket), _in(base1, _nc(la) * _nc(lb) * nket), _in(Rx, 3)
    _lib.call("pcg_two_electron_hrr", _p(t), _p(b0), _p(b1), _p(rx), la, lb, lc, ld, goofy)


def one_electron_fundamentals(fundamentals, sigma_P, U_P, P, Rc, Z, na, nb, m):
    na, nb, m = _int(na, nb, m)
    n = na * nb
    f = _out(fundamentals, (m + 1) * n)
    s, u, pp, rc = _in(sigma_P, n), _in(U_P, n), _in(P, 3 * n), _in(Rc, 3)
    _lib.call("pcg_one_electron_fundamentals", _p(f), _p(s), _p(u), _p(pp), _p(rc), float(Z), na, nb, m)


def _base_list(base_list, n_base):
    if not isinstance(base_list, (list, tuple)) or len(base_list) < n_base:
        raise TypeError(_PARSE)
    return [_in(b) for b in base_list[:n_base]]


def _ptr_array(arrs):
    return (_lib.P_DBL * len(arrs))(*[_p(a) for a in arrs])


def one_electron_vrr(target, base_list, sigma_P, P, Ra, Rc, atom_index, n_base, na, nb, la):
    atom_index, n_base, na, nb, la = _int(atom_index, n_base, na, nb, la)
    n = na * nb
    t = _out(target, _nc(la) * n)
    bl = _base_list(base_list, n_base)
    n1, n2 = _nc(la - 1) * n, _nc(la - 2) * n
    need = [n1] + ([n2] if atom_index == -1 else [n1, n2, n2])
    for b, k in zip(bl, need):
        if b.size < k:
            raise ValueError("base class array of %d elements, %d required" % (b.size, k))
    s, pp, ra = _in(sigma_P, n), _in(P, 3 * n), _in(Ra, 3)
    rc = np.zeros(3) if atom_index == -1 else _in(Rc, 3)
    _lib.call("pcg_one_electron_vrr", _p(t), _ptr_array(bl), _p(s), _p(pp), _p(ra), _p(rc), atom_index, n_base,
              na, nb, la)


def one_electron_hrr(target, base_list, Rab, n_base, na, nb, la, lb):
    n_base, na, nb, la, lb = _int(n_base, na, nb, la, lb)
    t = _out(target, _nc(la) * na * _nc(lb) * nb)
    bl = _base_list(base_list, n_base)
    if bl[0].size < _nc(la + 1) * na * _nc(lb - 1) * nb or bl[1].size < _nc(la) * na * _nc(lb - 1) * nb:
        raise ValueError("base class arrays too small")
    _lib.call("pcg_one_electron_hrr", _p(t), _ptr_array(bl), _p(_in(Rab, 3)), n_base, na, nb, la, lb)


def one_electron_kinetic(target, base_list, exB, n_base, na, nb, la, lb):
    n_base, na, nb, la, lb = _int(n_base, na, nb, la, lb)
    rows = _nc(la) * na
    t = _out(target, rows * _nc(lb) * nb)
    bl = _base_list(base_list, n_base)
    need = [rows * _nc(lb + 2) * nb, rows * _nc(lb) * nb, rows * _nc(lb - 2) * nb]
    for b, k in zip(bl, need):
        if b.size < k:
            raise ValueError("base class array of %d elements, %d required" % (b.size, k))
    _lib.call("pcg_one_electron_kinetic", _p(t), _ptr_array(bl), _p(_in(exB, nb)), n_base, na, nb, la, lb)


def one_electron_contract(target, base, cc, na, nb, la, lb):
    na, nb, la, lb = _int(na, nb, la, lb)
    t = _out(target, _nc(la) * _nc(lb))
    b, c = _in(base, _nc(la) * na * _nc(lb) * nb), _in(cc, na * nb)
    _lib.call("pcg_one_electron_contract", _p(t), _p(b), _p(c), na, nb, la, lb)
