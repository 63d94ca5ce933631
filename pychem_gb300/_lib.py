"""ctypes binding of libpychem_gb300.so (include/pychem_gb300.h).

The library is built in-tree by ``pychem_gb300.build``.  There is no fallback: if the
shared library is missing or no CUDA device is present, every entry point raises.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libpychem_gb300.so")

c_int, c_double, c_void_p, c_longlong = ctypes.c_int, ctypes.c_double, ctypes.c_void_p, ctypes.c_longlong
P_INT = ctypes.POINTER(ctypes.c_int)
P_DBL = ctypes.POINTER(ctypes.c_double)
P_FLT = ctypes.POINTER(ctypes.c_float)
P_LL = ctypes.POINTER(ctypes.c_longlong)
PP_DBL = ctypes.POINTER(P_DBL)


class PcgError(RuntimeError):
    pass


class BasisT(ctypes.Structure):
    _fields_ = [("nshell", c_int), ("nprim", c_int), ("natom", c_int), ("nbf", c_int),
                ("sh_l", c_void_p), ("sh_nprim", c_void_p), ("sh_prim", c_void_p), ("sh_ao", c_void_p),
                ("sh_atom", c_void_p), ("sh_xyz", c_void_p), ("pr_exp", c_void_p), ("pr_cc", c_void_p),
                ("at_xyz", c_void_p), ("at_z", c_void_p), ("ld", c_int), ("sh_blk", c_void_p), ("sh_at0", c_void_p),
                ("sh_nat", c_void_p)]


class PairsT(ctypes.Structure):
    _fields_ = [("npair", c_int), ("npp", c_int), ("A", c_void_p), ("B", c_void_p), ("ppoff", c_void_p),
                ("npp_of", c_void_p), ("AB", c_void_p), ("zeta", c_void_p), ("P", c_void_p), ("PA", c_void_p),
                ("K", c_void_p), ("oo2z", c_void_p), ("Kf", c_void_p), ("ao4", c_void_p),
                ("pf8", c_void_p)]


# name -> argtypes (all return int status unless listed in _RESTYPES)
_SIGS = {
    "pcg_version": [],
    "pcg_last_error": [],
    "pcg_device_init": [],
    "pcg_shellpair_quantities": [P_DBL, P_DBL, P_DBL, P_DBL, P_DBL, c_int, P_DBL, P_DBL, c_int],
    "pcg_two_electron_bound": [P_DBL, P_DBL, P_DBL, c_int, c_int, c_int, c_int],
    "pcg_two_electron_fundamentals": [P_DBL] * 8 + [c_int] * 6 + [c_double],
    "pcg_two_electron_vrr": [P_DBL] * 11 + [c_int] * 7,
    "pcg_two_electron_contract": [P_DBL] * 4 + [c_int] * 6,
    "pcg_two_electron_hrr": [P_DBL] * 4 + [c_int] * 5,
    "pcg_one_electron_fundamentals": [P_DBL] * 5 + [c_double, c_int, c_int, c_int],
    "pcg_one_electron_vrr": [P_DBL, PP_DBL, P_DBL, P_DBL, P_DBL, P_DBL] + [c_int] * 5,
    "pcg_one_electron_hrr": [P_DBL, PP_DBL, P_DBL] + [c_int] * 5,
    "pcg_one_electron_kinetic": [P_DBL, PP_DBL, P_DBL] + [c_int] * 5,
    "pcg_one_electron_contract": [P_DBL, P_DBL, P_DBL] + [c_int] * 4,
    "pcg_pair_data": [ctypes.POINTER(BasisT), c_int] + [c_void_p] * 10 + [c_void_p],
    "pcg_pair_data_f32": [c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p],
    "pcg_pair_ao": [ctypes.POINTER(BasisT), c_int, c_void_p, c_void_p, c_void_p, c_void_p],
    "pcg_one_electron": [ctypes.POINTER(BasisT), c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p],
    "pcg_eri_class_id": [c_int] * 4,
    "pcg_eri_class_nout": [c_int],
    "pcg_eri_class": [c_int, ctypes.POINTER(BasisT), ctypes.POINTER(PairsT), c_void_p, c_int, c_void_p, c_int,
                      c_void_p],
    "pcg_schwarz_class": [c_int, c_void_p, c_int, c_void_p, c_void_p, c_void_p],
    "pcg_expand_tasks": [c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_longlong, c_void_p, c_void_p],
    "pcg_digest_class": [c_int, ctypes.POINTER(BasisT), ctypes.POINTER(PairsT), c_void_p, c_int, c_void_p,
                         c_void_p, c_void_p, c_void_p],
    "pcg_digest_class_u": [c_int, ctypes.POINTER(BasisT), ctypes.POINTER(PairsT), c_void_p, c_int, c_void_p, c_void_p,
                           c_void_p, c_void_p, c_void_p, c_void_p, c_void_p],
    "pcg_scattering_class": [c_int, ctypes.POINTER(BasisT), ctypes.POINTER(PairsT), c_void_p, c_int,
                             ctypes.c_double, c_void_p, c_void_p],
    "pcg_digest_class_co": [c_int, ctypes.POINTER(BasisT), ctypes.POINTER(PairsT), c_void_p, c_int, c_void_p, c_int,
                            c_void_p, c_void_p, c_void_p, c_void_p],
    "pcg_fock_build": [c_int, c_void_p, c_void_p, c_void_p, c_void_p],
    "pcg_fock_build_batched": [c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p],
    "pcg_dense_class": [c_int, ctypes.POINTER(BasisT), ctypes.POINTER(PairsT), c_void_p, c_int, c_void_p,
                        c_void_p, c_void_p],
    "pcg_fma_probe": [c_int, c_int, c_int, c_int, c_void_p, c_void_p],
    "pcg_mlp_gemm": [c_int, c_int, c_int, c_void_p, c_longlong, c_longlong, c_void_p, c_int, c_longlong, c_longlong,
                     c_void_p, c_int, c_int, c_void_p, c_void_p, c_int, c_void_p],
    "pcg_mlp_dsilu": [c_longlong, c_void_p, c_void_p, c_void_p],
    "pcg_mlp_colsum": [c_int, c_int, c_void_p, c_void_p, c_void_p],
    "pcg_mlp_mse": [c_longlong, c_void_p, c_void_p, c_void_p, ctypes.c_float, c_void_p, c_void_p, c_void_p],
    "pcg_mlp_adam": [c_longlong, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, ctypes.c_float, ctypes.c_float,
                     ctypes.c_float, ctypes.c_float, c_int, c_void_p],
    "pcg_jacobi_eigh": [c_int, c_int, c_void_p, c_void_p, c_void_p, c_int, c_void_p, c_int, c_double, c_void_p,
                        c_void_p],
    "pcg_dense_pairs_class": [c_int, ctypes.POINTER(BasisT), ctypes.POINTER(PairsT), c_void_p, c_int, c_void_p,
                              c_void_p, c_void_p, c_void_p],
    "pcg_sym_pairs_class": [c_int, ctypes.POINTER(BasisT), ctypes.POINTER(PairsT), c_void_p, c_int, c_void_p,
                            c_void_p, c_longlong, c_void_p, c_void_p],
    "pcg_mark_pairs": [c_void_p, c_int, c_void_p, c_void_p],
    "pcg_pair_colmap": [c_int, c_void_p, c_void_p, c_void_p],
    "pcg_unpack_pairs": [c_longlong, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p],
    "pcg_dgemm": [c_int, c_int, c_int, c_int, c_double, c_void_p, c_longlong, c_longlong, c_longlong, c_void_p,
                  c_longlong, c_longlong, c_longlong, c_double, c_void_p, c_longlong, c_longlong, c_longlong, c_void_p],
    "pcg_oa_correction": [c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p],
    "pcg_diis_step": [c_longlong, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                      c_void_p, c_void_p, c_void_p],
    "pcg_mp2_pair_sums": [c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p],
    "pcg_ozaki_tc_workspace": [c_int, c_int, c_int],
    "pcg_ozaki_gemm_tc": [c_longlong, c_int, c_int, c_void_p, c_longlong, c_void_p, c_longlong, c_longlong, c_void_p,
                          c_longlong, c_longlong, c_int, c_int, c_void_p, ctypes.c_size_t, c_void_p],
    "pcg_ozaki_tc_status": [c_void_p, c_void_p],
    "pcg_fock_build_noalloc": [ctypes.POINTER(BasisT), ctypes.POINTER(PairsT), c_int, c_void_p, c_void_p, c_void_p,
                               c_void_p, c_void_p, c_void_p, c_void_p, c_void_p],
}
# entry points that launch exactly one kernel of this library per call
LAUNCHERS = {"pcg_pair_data", "pcg_pair_data_f32", "pcg_pair_ao", "pcg_one_electron", "pcg_eri_class", "pcg_schwarz_class", "pcg_expand_tasks",
             "pcg_digest_class", "pcg_digest_class_u", "pcg_digest_class_co", "pcg_scattering_class", "pcg_fock_build", "pcg_fock_build_batched", "pcg_dense_class", "pcg_fma_probe", "pcg_jacobi_eigh", "pcg_dense_pairs_class", "pcg_sym_pairs_class", "pcg_mark_pairs", "pcg_pair_colmap", "pcg_unpack_pairs",
             "pcg_dgemm", "pcg_oa_correction", "pcg_mp2_pair_sums", "pcg_mlp_gemm", "pcg_mlp_dsilu",
             "pcg_mlp_colsum", "pcg_mlp_mse", "pcg_mlp_adam",
             "pcg_shellpair_quantities", "pcg_two_electron_bound", "pcg_two_electron_fundamentals",
             "pcg_two_electron_vrr", "pcg_two_electron_contract", "pcg_two_electron_hrr",
             "pcg_one_electron_fundamentals", "pcg_one_electron_vrr", "pcg_one_electron_hrr",
             "pcg_one_electron_kinetic", "pcg_one_electron_contract"}
launch_count = 0
_RESTYPES = {"pcg_last_error": ctypes.c_char_p, "pcg_ozaki_tc_workspace": ctypes.c_size_t}
# entry points that launch more than one kernel of this library per call
MULTI_LAUNCH = {"pcg_ozaki_gemm_tc": 2, "pcg_diis_step": 4}

_lib = None


def exported_symbols():
    return sorted(_SIGS)


def load(path=None):
    """Load the shared library (no CUDA call is made)."""
    global _lib
    if _lib is None:
        p = path or LIB_PATH
        if not os.path.exists(p):
            raise PcgError("libpychem_gb300.so not built (run: python -m pychem_gb300.build)")
        L = ctypes.CDLL(p)
        for name, argt in _SIGS.items():
            fn = getattr(L, name)
            fn.argtypes = argt
            fn.restype = _RESTYPES.get(name, c_int)
        _lib = L
    return _lib


def check(rc, what=""):
    if rc != 0:
        msg = load().pcg_last_error()
        raise PcgError("%s failed (status %d): %s" % (what, rc, msg.decode() if msg else ""))


def call(name, *args):
    global launch_count
    if name in LAUNCHERS:
        launch_count += 1
    launch_count += MULTI_LAUNCH.get(name, 0)
    rc = getattr(load(), name)(*args)
    check(rc, name)
    return rc
