"""Recorded ``_c_ints`` calls of the upstream scattering-integral path.

Run once where the reference tree is present, its path in the environment
variable ``PYCHEM_REFERENCE`` (required):

    python tests/golden/make_golden_c_ints_scattering.py

Records every ``_c_ints`` call (inputs and in-place outputs) that
``Methods/integrals.py:two_electron`` makes with ``ints_type = 1`` -- the j0(S r12)
fundamentals of ``Methods/c_ints/two_electron_scattering.c`` and the shared VRR,
contraction and HRR steps -- for shell quartets of water / cc-pVDZ with a hydrogen
atom 30 bohr away, at momentum transfers that reach every regime of
``spherical_bessel_j.c`` (S = 0, R = 0, series, upward recursion, asymptotic form).
Writes ``c_ints_scattering_calls.{npz,json}`` in the layout of ``c_ints_calls``.
"""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import make_golden  # noqa: E402
import refrun  # noqa: E402


def main():
    root = refrun.prepare()
    ns = refrun.load(root)
    import Methods
    rec = make_golden.Recorder([ns["c_ints"], Methods._c_ints], per_func=100)
    atoms = make_golden.water() + [["H", 1.0, 0.0, 0.0, 15.875]]      # about 30 bohr away
    mol, st = refrun.molecule_from_spec(ns, atoms, "cc-pVDZ", multiplicity=2, reference="UHF")
    sp = mol.ShellPairs
    far = mol.NCgtf - 3          # first shell of the distant hydrogen (s, s, p)
    quartets = [((0, 0), (0, 0)), ((3, 5), (6, 8)), ((5, 5), (5, 5)), ((0, 3), (far, far)),
                ((3, 3), (far, far + 1)), ((6, 8), (far, far))]
    for S in (0.0, 0.4, 3.0, 7.5):
        for bra, ket in quartets:
            ns["integrals"].two_electron(sp[bra], sp[ket], 1, S)
    rec.restore()
    rec.save(os.path.join(HERE, "c_ints_scattering_calls"))


if __name__ == "__main__":
    main()
