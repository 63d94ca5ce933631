"""Oracle energies of the two large benchmark configurations, for the GPU parity tests.

    python tests/golden/make_golden_configs.py [c2] [c3]

Writes ``configs.json`` (small, committed).  The reference itself cannot run these
sizes (its dense N^4 tensor would be 15 GB and 63 GB, its MP2 is O(N^6) Python), so
the values come from the CPU oracle (``oracle/oracle.py``), which is pinned to the
reference's own outputs on smaller molecules (``tests/test_oracle_golden.py``), here
over its packed store (``oracle.PackedStore``: the screened unique quartets, the
Coulomb/exchange contraction and the first MP2 quarter transform in threaded C, the
rest in NumPy) so that no dense tensor is formed:

* c2: (H2O)16 on a 4x2x2 grid, 2.9 A spacing, seeded rotations and N(0, 0.05 A)
  jitter (seed 2026), 6-31G, 208 AO: RHF total energy and RMP2 correlation energy;
* c3: all-trans C12H26, N(0, 0.03 A) jitter (seed 2026), cc-pVDZ, 298 AO: RHF total
  energy.

SCF: the oracle's consistent Pulay SCF from the core guess, |dE| < 1e-10 and D-RMS
< 1e-8, the upstream Schwarz rule (1e-8) and linear-dependence cut (1e-6).
Coordinates are stored in bohr, as used.
"""
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from oracle import oracle as O  # noqa: E402
from pychem_gb300 import workloads as W  # noqa: E402

OUT = os.path.join(HERE, "configs.json")
SEED = 2026


def case(name, coords_ang, basis, mp2):
    atoms = [(a[0], a[1], a[2] * O.TO_BOHR, a[3] * O.TO_BOHR, a[4] * O.TO_BOHR) for a in coords_ang]
    b = O.Basis(atoms, basis)
    t0 = time.time()
    S, H = b.one_electron()
    store = O.PackedStore(b)
    t1 = time.time()
    nocc = b.nelectrons() // 2
    r = O.rhf(S, H, None, nocc, b.nuclear_repulsion(), store=store)
    t2 = time.time()
    out = {"basis": basis, "nbf": b.nbf, "nocc": nocc, "atoms_bohr": [list(a) for a in atoms],
           "quartets": store.nquartets, "E_rhf": r["E"], "scf_iterations": r["iterations"],
           "converged": bool(r["converged"]), "seconds": {"integrals": t1 - t0, "scf": t2 - t1}}
    if mp2:
        out["E_mp2_corr"] = O.rmp2_packed(r["C"], r["eps"], store, nocc)
        out["seconds"]["mp2"] = time.time() - t2
    print(name, {k: v for k, v in out.items() if k != "atoms_bohr"}, flush=True)
    return out


def main(which):
    data = json.load(open(OUT)) if os.path.exists(OUT) else {}
    if "c2" in which:
        data["c2_water16_631g"] = case("c2", W.water_cluster(seed=SEED), "6-31G", mp2=True)
    if "c3" in which:
        data["c3_c12h26_ccpvdz"] = case("c3", W.alkane(12, seed=SEED), "cc-pVDZ", mp2=False)
    with open(OUT, "w") as fh:
        json.dump(data, fh, indent=1)


if __name__ == "__main__":
    main(sys.argv[1:] or ["c2", "c3"])
