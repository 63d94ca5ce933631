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
