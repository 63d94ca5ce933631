"""Extract the basis sets this package ships from the upstream basis library.

The numbers are published Gaussian basis-set data (exponents and contraction
coefficients); parity with the upstream code needs them bit-identical, so they are
read once from the upstream dict literal ``Data/basis.py:1`` (``get[BASIS][EL] =
[[l, [exp, cc], ...], ...]``) and written to ``basis_sets.json`` beside this file.

    python pychem_gb300/data/extract_basis.py [path-to-reference]
"""
import ast
import json
import os
import sys

SETS = ["STO3G", "321G", "631G", "631GS", "631GSS", "6311G", "CCPVDZ"]
ELEMENTS = ["H", "HE", "LI", "BE", "B", "C", "N", "O", "F", "NE",
            "NA", "MG", "AL", "SI", "P", "S", "CL", "AR"]


def main(ref):
    with open(os.path.join(ref, "Data", "basis.py")) as fh:
        tree = ast.parse(fh.read())
    lib = ast.literal_eval(tree.body[0].value)
    out = {}
    for name in SETS:
        out[name] = {el: lib[name][el] for el in ELEMENTS if el in lib[name]}
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "basis_sets.json")
    with open(path, "w") as fh:
        json.dump(out, fh, separators=(",", ":"))
    print("wrote", path, {k: len(v) for k, v in out.items()})


if __name__ == "__main__":
    src = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PYCHEM_REFERENCE")
    if not src:
        sys.exit("usage: extract_basis.py <reference tree>  (or set PYCHEM_REFERENCE)")
    main(src)
