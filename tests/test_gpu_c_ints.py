"""The drop-in `_c_ints` layer replays calls recorded from the upstream extension.

tests/golden/c_ints_calls.{json,npz} hold inputs and outputs of the upstream
functions captured while integrals.one_electron / two_electron ran on H2O cc-pVDZ
(s, p and d shells).  Each call is replayed through pychem_gb300._c_ints (one GPU
kernel per call, through the C ABI) and its in-place outputs compared.  Outputs that
depend on the Boys function differ from upstream only by the regenerated table's
interpolation error (~1e-12 relative); the bar is 1e-10.
"""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def load_calls(golden_dir):
    with open(os.path.join(golden_dir, "c_ints_calls.json")) as fh:
        manifest = json.load(fh)
    arrays = np.load(os.path.join(golden_dir, "c_ints_calls.npz"))
    return manifest, arrays


def build_args(call, arrays):
    args = []
    for kind, val in call["args"]:
        if kind == "array":
            args.append(arrays[val].copy())
        elif kind == "list":
            items = [arrays[k].copy() for k in val]
            if items and all(x.ndim == 0 for x in items):
                args.append(np.array([float(x) for x in items]))
            else:
                args.append(items)
        elif kind == "float":
            args.append(float(val))
        else:
            args.append(int(val))
    return args


def test_replay_recorded_calls(golden_dir):
    from pychem_gb300 import _c_ints
    manifest, arrays = load_calls(golden_dir)
    seen = set()
    for k, call in enumerate(manifest):
        args = build_args(call, arrays)
        getattr(_c_ints, call["fn"])(*args)
        for idx, key in call["outputs"]:
            ref = arrays[key]
            got = np.asarray(args[idx])
            scale = max(1.0, float(np.abs(ref).max()))
            assert np.abs(got - ref).max() <= 1e-10 * scale, (k, call["fn"], float(np.abs(got - ref).max()))
        seen.add(call["fn"])
    assert len(seen) == 11, sorted(seen)


def test_error_behaviour():
    from pychem_gb300 import _c_ints
    with pytest.raises(TypeError):
        _c_ints.two_electron_bound(np.zeros(1, dtype=np.float32), np.ones((1, 1)), np.ones((1, 1)), 1, 1, 1, 1)
    with pytest.raises(ValueError):
        _c_ints.two_electron_bound(np.zeros(4), np.ones((1, 1)), np.ones((1, 1)), 2, 2, 1, 1)
    from pychem_gb300._lib import PcgError
    with pytest.raises(PcgError):
        z = np.ones((1, 1))
        _c_ints.two_electron_fundamentals(np.zeros((1, 1, 1)), z, z, np.zeros((1, 1, 3)), z, z, np.zeros((1, 1, 3)),
                                          np.zeros((1, 1, 3)), 1, 1, 1, 1, 0, 1, -0.5)


def test_replay_recorded_scattering_calls(golden_dir):
    """Calls recorded from the upstream extension while integrals.two_electron ran with
    ints_type = 1 (make_golden_c_ints_scattering.py): the j0(S r12) fundamentals in
    every regime of the Bessel scheme, and the VRR, contraction and HRR steps that
    follow them."""
    from pychem_gb300 import _c_ints
    with open(os.path.join(golden_dir, "c_ints_scattering_calls.json")) as fh:
        manifest = json.load(fh)
    arrays = np.load(os.path.join(golden_dir, "c_ints_scattering_calls.npz"))
    nfund = 0
    for k, call in enumerate(manifest):
        args = build_args(call, arrays)
        getattr(_c_ints, call["fn"])(*args)
        for idx, key in call["outputs"]:
            ref = arrays[key]
            got = np.asarray(args[idx])
            scale = max(1.0, float(np.abs(ref).max()))
            assert np.abs(got - ref).max() <= 1e-12 * scale, (k, call["fn"], float(np.abs(got - ref).max()))
        nfund += call["fn"] == "two_electron_fundamentals"
    assert nfund == 24
