"""Run one phase of a benchmark workload, for profiling (ncu) on a bounded case.

    python -m pychem_gb300.profile_case --case water16 --phase eri [--repeat 2]

cases:  water16 ((H2O)16 / 6-31G, 208 AO), water8 ((H2O)8, 104 AO), water4 ((H2O)4),
        alkane12 (C12H26 / cc-pVDZ, 298 AO), ensemble (256 perturbed small molecules,
        6-31G, batched), mlp (the learned-guess network on 65,536 pairs), gemm (one
        tensor-core Ozaki GEMM of the first MP2 transform's shape: 77,824 rows of 208
        FP64 values (130 MB, more than L2) times 208 x 80)
phases: eri (ERI pass), fock (one Fock build), scf (full RHF), mp2 (RHF + MP2),
        mp2only (one RHF before the repeats, then MP2 alone per repeat);
        scattering (one j0(S r12) grid value at --S: Schwarz pass, quartet plan,
        integral store, contraction with the RHF densities, each timed);
        noci (the CI matrix of C2 / cc-pVDZ spin-flip doubles with CISD, 27
        determinants; --case is ignored); codensity (J/K of 756 random non-symmetric
        co-densities of C2 / cc-pVDZ in one pcg_digest_class_co pass per class, the
        NOCI digestion without the host's SVDs; --case is ignored);
        for mlp: train (forward, loss, backward, Adam); for gemm: tc
"""
import argparse
import time

import torch

from . import workloads as W
from .engine import GpuEngine
from .molecule import Molecule
from .scf import rhf, rmp2

CASES = {
    "water16": lambda: Molecule(W.water_cluster(), "6-31G"),
    "water8": lambda: Molecule(W.water_cluster(nx=2, ny=2, nz=2), "6-31G"),
    "water4": lambda: Molecule(W.water_cluster(nx=2, ny=2, nz=1), "6-31G"),
    "alkane12": lambda: Molecule(W.alkane(12), "cc-pVDZ"),
}


def codensity_case(args):
    """J/K of 756 random non-symmetric co-densities of C2 / cc-pVDZ (28 AO), one
    GpuEngine.coulomb_exchange call per repeat."""
    mol = Molecule([["C", 6.0, 0.0, 0.0, 0.0], ["C", 6.0, 1.25, 0.0, 0.0]], "cc-pVDZ")
    eng = GpuEngine(mol).prepare()
    g = torch.Generator(device="cuda").manual_seed(4)
    W = torch.randn(756, eng.nbf, eng.nbf, dtype=torch.float64, device="cuda", generator=g) * 0.05
    eng.coulomb_exchange(W)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.repeat):
        eng.coulomb_exchange(W)
    torch.cuda.synchronize()
    print("codensity C2 cc-pVDZ: 756 co-densities, %.3f ms per J/K pass" % ((time.perf_counter() - t0) * 1e3 / args.repeat))


def gemm_case(args):
    """One pcg_ozaki_gemm_tc of the first MP2 quarter transform's shape per repeat."""
    from .scf import ozaki_gemm_tc, ozaki_tc_status
    M, N, K = 128 * 152 * 4, 80, 208
    g = torch.Generator(device="cuda").manual_seed(1)
    X = torch.randn(M, K, dtype=torch.float64, device="cuda", generator=g)
    Y = torch.randn(K, N, dtype=torch.float64, device="cuda", generator=g)
    C = torch.empty(N * M, dtype=torch.float64, device="cuda")
    ozaki_gemm_tc(X, Y, C, M, N, K, K, (N, 1), (1, M))
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.repeat):
        ozaki_gemm_tc(X, Y, C, M, N, K, K, (N, 1), (1, M))
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.repeat
    flops = 21 * 2.0 * M * N * K
    print("tc gemm %d x %d x %d: %.3f ms per launch, %.1f TFLOP/s of digit-slice products, error flag %d"
          % (M, N, K, ms, flops / ms / 1e9, ozaki_tc_status("cuda")))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--case", default="water16", choices=sorted(CASES) + ["ensemble", "mlp", "gemm"])
    ap.add_argument("--phase", default="eri", choices=["eri", "fock", "scf", "mp2", "mp2only", "train", "scattering", "noci", "tc", "codensity"])
    ap.add_argument("--S", type=float, default=2.0)
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--repeat", type=int, default=1)
    args = ap.parse_args()
    if args.case == "ensemble":
        return ensemble_case(args)
    if args.case == "mlp":
        return mlp_case(args)
    if args.case == "gemm":
        return gemm_case(args)
    if args.phase == "noci":
        return noci_case(args)
    if args.phase == "codensity":
        return codensity_case(args)
    mol = CASES[args.case]()
    if args.phase == "scattering":
        return scattering_case(args, mol)
    eng = GpuEngine(mol, precision=args.precision)
    eng.one_electron(); eng.schwarz(); eng.build_tasks(); eng.compute_eris()
    if args.phase == "mp2only":
        r0 = rhf(eng)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.repeat):
        if args.phase == "mp2only":
            rmp2(eng, r0.C, r0.eps)
        elif args.phase == "eri":
            eng.compute_eris()
        elif args.phase == "fock":
            n = eng.nbf
            eng.fock(torch.eye(n, dtype=torch.float64, device="cuda") * 0.1)
        elif args.phase == "scf":
            r = rhf(eng)
        else:
            r = rhf(eng)
            rmp2(eng, r.C, r.eps)
    torch.cuda.synchronize()
    print("%s %s %s: %.4f s per repeat, %d quartets" % (args.case, args.phase, args.precision,
                                                         (time.perf_counter() - t0) / args.repeat,
                                                         eng.stats["quartets"]))


def ensemble_case(args):
    from .ensemble import EnsembleEngine, rhf_batched
    mols = [Molecule(c, "6-31G") for c in W.ensemble(n=256, seed=2026)]
    eng = EnsembleEngine(mols, precision=args.precision).prepare()
    if args.phase == "mp2only":
        r0 = rhf(eng)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.repeat):
        if args.phase == "mp2only":
            rmp2(eng, r0.C, r0.eps)
        elif args.phase == "eri":
            eng.compute_eris()
        else:
            r = rhf_batched(eng)
    torch.cuda.synchronize()
    print("ensemble %s: %.4f s per repeat, %d molecules" % (args.phase, (time.perf_counter() - t0) / args.repeat,
                                                           eng.B))


def mlp_case(args):
    from .learned.blocks import NFEAT, NPARAM
    from .learned.mlp import PairMLP
    net = PairMLP(seed=0)
    g = torch.Generator(device="cuda").manual_seed(0)
    X = torch.randn(65536, NFEAT, device="cuda", generator=g)
    T = torch.randn(65536, NPARAM, device="cuda", generator=g)
    M = torch.ones_like(T)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.repeat):
        Y, cache = net.forward(X, keep=True)
        loss, dY = net.loss_grad(Y, T, M)
        net.adam(net.backward(dY, cache), 1e-3)
    torch.cuda.synchronize()
    print("mlp train step: %.4f s per repeat" % ((time.perf_counter() - t0) / args.repeat))



def _timed(fn):
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out = fn()
    torch.cuda.synchronize()
    return out, time.perf_counter() - t0


def scattering_case(args, mol):
    """One grid value of the scattering intensity, phase by phase."""
    r = rhf(GpuEngine(mol).prepare())
    eng = GpuEngine(mol)
    eng.one_electron()
    for k in range(args.repeat + 1):
        eng.scattering = args.S
        _, t_q = _timed(eng.schwarz)
        _, t_p = _timed(eng.build_tasks)
        _, t_e = _timed(eng.compute_eris)
        (Fa, Fb), t_c = _timed(lambda: eng.fock_u(r.D, r.D))
        if k:
            print("%s scattering S=%.2f: schwarz %.4f s, plan %.4f s, integrals %.4f s (%d quartets), "
                  "contraction %.4f s" % (args.case, args.S, t_q, t_p, t_e, eng.stats["quartets"], t_c))


def noci_case(args):
    """The CI matrix of spin-flip NOCI on C2 / cc-pVDZ (SFD-CISD)."""
    from . import noci
    mol = Molecule([["C", 6.0, 0.0, 0.0, 0.0], ["C", 6.0, 1.25, 0.0, 0.0]], "cc-pVDZ")
    eng = GpuEngine(mol).prepare()
    out = noci.run(eng, "SFD-CISD", reference="UHF", constrain_excited=True)
    na, nb = mol.NAlphaElectrons, mol.NBetaElectrons
    for _ in range(args.repeat + 1):
        _, t = _timed(lambda: noci.noci_matrix(eng, out["dets_alpha"], out["dets_beta"], na, nb))
    print("noci C2 cc-pVDZ SFD-CISD: %d determinants, CI matrix %.4f s" % (len(out["dets_alpha"]), t))


if __name__ == "__main__":
    main()
