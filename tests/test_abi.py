"""The C-ABI library loads (no GPU needed) and exports every function that
include/*.h declares; the ctypes binding covers the same set."""
import glob
import os
import re

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    names = set()
    for h in glob.glob(os.path.join(REPO, "include", "*.h")):
        text = re.sub(r"/\*.*?\*/", "", open(h).read(), flags=re.S)
        names.update(re.findall(r"\b(pcg_\w+)\s*\(", text))
    return names


@pytest.fixture(scope="module")
def lib():
    from pychem_gb300 import _lib, build
    if not os.path.exists(_lib.LIB_PATH):
        build.build()
    return _lib.load()


def test_every_declared_symbol_is_exported(lib):
    names = declared()
    assert len(names) >= 25
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_matches_header():
    from pychem_gb300 import _lib
    assert declared() == set(_lib.exported_symbols())


def test_cpu_only_calls(lib):
    # pure host functions: no CUDA context needed
    assert lib.pcg_version() == 1
    assert lib.pcg_eri_class_id(1, 1, 1, 1) == 5
    assert lib.pcg_eri_class_id(0, 1, 0, 0) == -1
    assert lib.pcg_eri_class_nout(20) == 625


def test_generated_header_is_current():
    import subprocess
    import sys
    r = subprocess.run([sys.executable, os.path.join(REPO, "pychem_gb300", "csrc", "gen_eri.py"), "--check"])
    assert r.returncode == 0


def test_noalloc_fock_rejects_bad_layout_before_any_cuda_call(lib):
    # pcg_fock_build_noalloc checks its arguments before its first CUDA call, so these
    # calls run without a GPU: a row stride other than nbf would index past the
    # cleared part of the static accumulator, and a bad class entry must be refused
    # before anything is queued.
    import ctypes
    from pychem_gb300._lib import BasisT, PairsT
    fake = ctypes.c_void_p(16)          # never dereferenced: every call below is rejected
    b, p = BasisT(), PairsT()
    b.nbf, b.ld = 100, 101
    assert lib.pcg_fock_build_noalloc(ctypes.byref(b), ctypes.byref(p), 0, None, None, None, None,
                                      fake, fake, fake, None) == 2
    assert b"ld must be 0 or nbf" in lib.pcg_last_error()
    b.ld = 100
    cls = (ctypes.c_int * 2)(0, 21)
    ntask = (ctypes.c_int * 2)(1, 1)
    ptrs = (ctypes.c_void_p * 2)(16, 16)
    assert lib.pcg_fock_build_noalloc(ctypes.byref(b), ctypes.byref(p), 2, ctypes.cast(cls, ctypes.c_void_p),
                                      ctypes.cast(ptrs, ctypes.c_void_p), ctypes.cast(ntask, ctypes.c_void_p),
                                      ctypes.cast(ptrs, ctypes.c_void_p), fake, fake, fake, None) == 2
    assert b"bad class entry 1" in lib.pcg_last_error()


def test_mp2_entry_points_reject_bad_arguments_before_any_cuda_call(lib):
    # the compact-pair and pair-sum entry points of the MP2 path check their
    # arguments first, so these refused calls need no GPU
    import ctypes
    from pychem_gb300._lib import BasisT, PairsT
    fake = ctypes.c_void_p(16)          # never dereferenced: every call below is rejected
    assert lib.pcg_mp2_pair_sums(0, 4, fake, fake, fake, fake, None) == 2
    assert b"pcg_mp2_pair_sums" in lib.pcg_last_error()
    assert lib.pcg_mp2_pair_sums(4, 4, None, fake, fake, fake, None) == 2
    assert lib.pcg_mark_pairs(fake, 10, None, None) == 2
    assert lib.pcg_mark_pairs(None, 10, fake, None) == 2
    assert lib.pcg_pair_colmap(0, None, fake, None) == 2
    assert lib.pcg_pair_colmap(8, None, None, None) == 2
    assert lib.pcg_unpack_pairs(4, 8, 36, None, fake, fake, None) == 2
    assert b"pcg_unpack_pairs" in lib.pcg_last_error()
    b, p = BasisT(), PairsT()
    assert lib.pcg_sym_pairs_class(0, ctypes.byref(b), ctypes.byref(p), fake, 1, fake, None, 10, fake, None) == 2
    assert lib.pcg_sym_pairs_class(0, ctypes.byref(b), ctypes.byref(p), fake, 1, fake, fake, 0, fake, None) == 2
    assert lib.pcg_sym_pairs_class(21, ctypes.byref(b), ctypes.byref(p), fake, 1, fake, fake, 10, fake, None) == 2


def _declared_arities():
    """name -> number of parameters of every pcg_* prototype in include/*.h."""
    out = {}
    for h in glob.glob(os.path.join(REPO, "include", "*.h")):
        text = re.sub(r"/\*.*?\*/", "", open(h).read(), flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        for m in re.finditer(r"\b(pcg_\w+)\s*\(([^;{]*?)\)\s*;", text, flags=re.S):
            params = m.group(2).strip()
            out[m.group(1)] = 0 if params in ("", "void") else params.count(",") + 1
    return out


def test_binding_arities_match_the_prototypes():
    # the ctypes argument lists of pychem_gb300/_lib.py have as many entries as the
    # header's prototypes have parameters (a drift here would pass wrong arguments)
    from pychem_gb300 import _lib
    ar = _declared_arities()
    assert len(ar) >= 25
    bad = {n: (ar[n], len(_lib._SIGS[n])) for n in ar if n in _lib._SIGS and ar[n] != len(_lib._SIGS[n])}
    assert not bad, bad


def test_binding_types_match_the_prototypes():
    # each ctypes argument type matches the C parameter type: pointers as pointers,
    # and int / long long / size_t / double / float by width (an int passed where the
    # prototype has long long would leave the upper half undefined)
    import ctypes
    from pychem_gb300 import _lib
    kinds = {"long long": ctypes.c_longlong, "size_t": ctypes.c_size_t, "double": ctypes.c_double,
             "float": ctypes.c_float, "int": ctypes.c_int}
    bad = []
    for h in glob.glob(os.path.join(REPO, "include", "*.h")):
        text = re.sub(r"/\*.*?\*/", "", open(h).read(), flags=re.S)
        for m in re.finditer(r"\b(pcg_\w+)\s*\(([^;{]*?)\)\s*;", text, flags=re.S):
            name, params = m.group(1), m.group(2).strip()
            if name not in _lib._SIGS or params in ("", "void"):
                continue
            for k, (p, t) in enumerate(zip(params.split(","), _lib._SIGS[name])):
                p = " ".join(p.replace("const", " ").split())
                if "*" in p:
                    ok = t in (ctypes.c_void_p, ctypes.c_char_p) or hasattr(t, "_type_") and t.__name__.startswith("LP_")
                else:
                    base = next((c for key, c in kinds.items() if p.startswith(key + " ") or p == key), None)
                    ok = base is not None and ctypes.sizeof(base) == ctypes.sizeof(t) and \
                        (base in (ctypes.c_double, ctypes.c_float)) == (t in (ctypes.c_double, ctypes.c_float))
                if not ok:
                    bad.append((name, k, p, t.__name__))
    assert not bad, bad
