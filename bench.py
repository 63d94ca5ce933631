"""Benchmark: plain-FP64 direct RHF + MP2 of a 16-water cluster in 6-31G on one GB300.

Workload (the configuration the headline metric is quoted on): (H2O)16 on a 4x2x2 grid
with 2.9 A spacing, seeded random rotations and N(0, 0.05 A) jitter, 6-31G, 208 AO,
80 doubly occupied orbitals (pychem_gb300.workloads.water_cluster, seed 2026).

One step = one complete solve from device-resident shells: primitive-pair data,
S/T/V, Schwarz pass, screened quartet lists, every screened ERI into the in-core
store, SCF to |dE| < 1e-10 Eh and D-RMS < 1e-8, then the MP2 AO->MO transform and
energy.  `value` is the time of that step (time-to-convergence incl. MP2, seconds,
CUDA events, L2 flushed between steps); `e2e` is the same solve through the public
call pychem_gb300.api.rhf_mp2 from host coordinates to host results.

Extra keys on the same line (rank 0, N = 1): ``mixed`` (mixed-precision ERIs on the
same workload), ``alkane_mixed`` (C12H26 / cc-pVDZ), ``ensemble`` (1024 molecules,
batched SCF), ``learned_guess`` (learned initial densities on 1024 held-out molecules),
``noci_spin_flip`` (spin-flip NOCI, C2 / cc-pVDZ, 27 determinants) and ``scattering``
(electron-scattering intensities, (H2O)8 / 6-31G, 16 grid values), each with the CPU
oracle's time on a bounded sample where it has one.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
"""
import argparse
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import tempfile
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "RHF time-to-convergence & ERI quartets/s on 1 GB300, learned/mixed vs plain FP64 @1e-8 Eh"
WORKLOAD = "(H2O)16 water cluster, 6-31G, 208 AO, RHF + MP2"
SEED = 2026


def env_rank():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def oracle_energies():
    """Oracle energies of the benchmark configurations (tests/golden/configs.json,
    made by tests/golden/make_golden_configs.py); {} when absent."""
    try:
        with open(os.path.join(REPO, "tests", "golden", "configs.json")) as fh:
            return json.load(fh)
    except OSError:
        return {}


def load_peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as fh:
            return json.load(fh)
    except OSError:
        return {}


# ------------------------------------------------------------------------------------
# CPU side (oracle port): shared by the cpu_baseline leg and the reference arm
# ------------------------------------------------------------------------------------
def _cpu_worker(args):
    atoms, basis, quads = args
    import ctypes
    import numpy as np
    from oracle import oracle as O
    b = O.Basis(atoms, basis)
    q = np.ascontiguousarray(np.asarray(quads, dtype=np.int32).reshape(-1))
    t0 = time.perf_counter()
    O.lib().oracle_eri_list(b.c, len(quads), q.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
    return time.perf_counter() - t0


_PLAN = {}


def cpu_plan(atoms, basis, rng):
    """Schwarz pass and screened-quartet count on the CPU oracle; returns
    (total screened quartets, sampler).  Cached per molecule."""
    import numpy as np
    from oracle import oracle as O
    key = (basis, tuple(tuple(a[2:]) for a in atoms))
    if key not in _PLAN:
        b = O.Basis(atoms, basis)
        Q = b.schwarz()
        ia, ib = np.triu_indices(b.nshell)
        q = Q[ia, ib]
        thr = O.INTEGRAL_THRESHOLD
        order = np.argsort(-q)
        qs = q[order]
        # row i (sorted order) pairs with j <= i when q_i q_j > thr, plus its own diagonal
        cpre = np.empty(len(qs), dtype=np.int64)
        for i in range(len(qs)):
            cpre[i] = min(i + 1, np.searchsorted(-qs[: i + 1] * qs[i], -thr, side="left"))
        cnt = cpre + (cpre <= np.arange(len(qs)))
        _PLAN[key] = (ia, ib, order, cpre, cnt, int(cnt.sum()))
    ia, ib, order, cpre, cnt, total = _PLAN[key]

    def sample(n):
        rows = rng.choice(len(cnt), size=n, p=cnt / total)
        j = (rng.random(n) * cnt[rows]).astype(np.int64)
        j = np.where(j >= cpre[rows], rows, j)
        p1, p2 = order[rows], order[j]
        return np.stack([ia[p1], ib[p1], ia[p2], ib[p2]], axis=1).astype(np.int32)
    return total, sample, None


def cpu_eri_rate(atoms, basis, workers, target_s=10.0, seed=SEED):
    """Screened quartets/s of the CPU oracle on a bounded random sample; returns
    (quartets_per_s, total_quartets, sample_description, cores)."""
    import numpy as np
    rng = np.random.default_rng(seed)
    total, sample, _ = cpu_plan(atoms, basis, rng)
    probe = sample(2000)
    t = _cpu_worker((atoms, basis, probe))
    per = t / len(probe)
    n = int(min(total, max(2000, target_s / per * workers)))
    quads = sample(n)
    if workers == 1:
        wall = _cpu_worker((atoms, basis, quads))
    else:
        chunks = [quads[k::workers] for k in range(workers)]
        ctx = mp.get_context("spawn")
        with ctx.Pool(workers) as pool:
            # each worker times its own kernel loop (process start-up excluded); the
            # slowest worker bounds the parallel wall time
            wall = max(pool.map(_cpu_worker, [(atoms, basis, c) for c in chunks]))
    rate = n / wall
    desc = "%d of %d screened shell quartets (uniform sample) through the C oracle port on %d core(s), %.1f s" % (
        n, total, workers, wall)
    return rate, total, desc


def cpu_full_estimate(atoms, basis, nocc, scf_iterations, threads, seed=SEED, target_s=3.0):
    """CPU time of the whole RHF + MP2 workload through the oracle port (the pinned
    restatement of the reference's integral, SCF and MP2 algorithms), on `threads`
    host threads, from bounded samples:
      ERIs: random windows of 512 consecutive screened quartets (threaded C blocks),
        scaled to every quartet;
      SCF: one Coulomb/exchange build over the sample's blocks, scaled to every
        quartet and to the oracle SCF's iteration count (tests/golden/configs.json);
      MP2: the first quarter transform (threaded C) over the sample for o_s
        occupied orbitals, scaled to every quartet and all nocc; the other three
        transforms (NumPy/BLAS) for one occupied orbital, times nocc.
    Returns (seconds, description, breakdown)."""
    import numpy as np
    from oracle import oracle as O
    rng = np.random.default_rng(seed)
    key = ("full", basis, tuple(tuple(a[2:]) for a in atoms))
    b = O.Basis(atoms, basis)
    if key not in _PLAN:
        _PLAN[key] = b.quartet_array()
    allq = _PLAN[key]
    total = len(allq)
    n = b.nbf
    win = 512

    def sample(m):
        # whole windows of the canonical quartet order, so that the sample keeps the
        # full run's locality (consecutive quartets share their bra pair)
        k = max(1, m // win)
        starts = rng.choice(max(1, total // win), size=min(k, max(1, total // win)), replace=False) * win
        return np.concatenate([allq[s0:s0 + win] for s0 in np.sort(starts)])

    probe = O.PackedStore(b, nthreads=threads, quads=sample(4096))
    t0 = time.perf_counter()
    O.PackedStore(b, nthreads=threads, quads=sample(4096))
    per = (time.perf_counter() - t0) / 4096
    quads = sample(int(min(total, max(4096, target_s / per))))
    nq = len(quads)
    t0 = time.perf_counter()
    st = O.PackedStore(b, nthreads=threads, quads=quads)
    t_eri = time.perf_counter() - t0
    M = rng.normal(size=(n, n))
    D = 0.01 * (M + M.T)
    t0 = time.perf_counter()
    st.jk(2.0 * D, D)
    t_jk = time.perf_counter() - t0
    o_s = max(1, min(nocc, threads))
    C = rng.normal(size=(n, nocc + 1))
    t0 = time.perf_counter()
    T1 = st.mp2_first_quarter(C[:, :o_s])
    t_q1 = time.perf_counter() - t0
    del probe
    # the other three transforms of one occupied orbital at full size (oracle.rmp2_packed)
    v = n - nocc
    Cv = rng.normal(size=(n, v))
    Co = rng.normal(size=(n, nocc))
    r_, s_ = np.tril_indices(n)
    T1i = rng.normal(size=(n, n * (n + 1) // 2))
    t0 = time.perf_counter()
    T2 = Cv.T @ T1i
    Mx = np.zeros((v, n, n))
    Mx[:, r_, s_] = T2
    Mx[:, s_, r_] = T2
    np.einsum("alk,lj,kb->ajb", Mx, Co, Cv, optimize=True)
    t_rest = time.perf_counter() - t0
    del T1, T1i, Mx
    scale = total / nq
    parts = {"eri_s": t_eri * scale, "scf_s": scf_iterations * t_jk * scale,
             "mp2_first_quarter_s": (nocc / o_s) * t_q1 * scale, "mp2_rest_s": nocc * t_rest}
    desc = ("oracle port on %d thread(s): %d of %d screened shell quartets (random windows of 512 consecutive quartets) for the ERI, Coulomb/exchange "
            "and first-MP2-transform kernels, scaled to every quartet, %d SCF iterations (the oracle SCF's own count) and "
            "%d occupied orbitals; the other MP2 transforms timed for one occupied orbital x %d; extrapolated"
            % (threads, nq, total, scf_iterations, nocc, nocc))
    return sum(parts.values()), desc, parts


def _c2_atoms_bohr():
    from pychem_gb300 import workloads as W
    return [(a[0], a[1], a[2] * 1.8897161646320724, a[3] * 1.8897161646320724, a[4] * 1.8897161646320724)
            for a in W.water_cluster(seed=SEED)]


def reference_arm(args):
    rank, world, _ = env_rank()
    if rank != 0:
        return
    from oracle import oracle as O
    O.build()
    atoms = _c2_atoms_bohr()
    ref = oracle_energies().get("c2_water16_631g", {})
    iters = int(ref.get("scf_iterations", 31))
    cores = os.cpu_count() or 1
    vals, desc, parts = [], "", {}
    for k in range(args.warmup + args.steps):
        v, desc, parts = cpu_full_estimate(atoms, "6-31G", 80, iters, cores, seed=SEED + k, target_s=1.0)
        if k >= args.warmup:
            vals.append(v)
    v = statistics.mean(vals)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": v * 1e3, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "basis": "6-31G", "seed": SEED},
            "cpu_baseline": {"value": v, "unit": "s", "cores": cores, "kind": "port", "sample": desc,
                             "breakdown_s": parts},
            "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


# ------------------------------------------------------------------------------------
# GPU arm
# ------------------------------------------------------------------------------------
class Clocks:
    def __init__(self, index):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.index = index
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=clocks.sm,clocks.max.sm,power.draw,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None
        return self

    def __exit__(self, *a):
        if self.p:
            self.p.terminate()
            self.p.wait()

    def summary(self):
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.strip()]
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[0])); mx.append(float(r[1]))
                for nm, v in zip(names, r[3:7]):
                    if v.strip().lower() == "active":
                        reasons.add(nm)
            except (ValueError, IndexError):
                pass
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def probe_peak(torch, _lib, fp32):
    import ctypes
    blocks, threads, iters = 152 * 8, 256, 4096
    out = torch.empty(blocks * threads, dtype=torch.float32 if fp32 else torch.float64, device="cuda")
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    best = 0.0
    for _ in range(4):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        _lib.call("pcg_fma_probe", blocks, threads, iters, 1 if fp32 else 0, ctypes.c_void_p(out.data_ptr()), s)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        best = max(best, blocks * threads * iters * 8 * 2 / (ms * 1e-3) / 1e12)
    return best


def ensemble_leg(torch, args, n=1024):
    """1024 perturbed H2O/NH3/CH4/HF/CH3OH/C2H6 (6-31G, 11-30 AO) in one batched SCF,
    against looping the one-molecule GPU SCF over a sample of the same ensemble.  Both
    sides are timed from Molecule objects to converged energies, host set-up included."""
    from pychem_gb300 import workloads as W
    from pychem_gb300.engine import GpuEngine
    from pychem_gb300.ensemble import EnsembleEngine, rhf_batched
    from pychem_gb300.molecule import Molecule
    from pychem_gb300.scf import rhf
    mols = [Molecule(c, "6-31G") for c in W.ensemble(n=n, seed=SEED)]
    times, dev_t, res, eng = [], [], None, None
    for k in range(args.warmup + max(1, args.steps)):
        del eng
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        eng = EnsembleEngine(mols)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        eng.prepare()
        res = rhf_batched(eng)
        e1.record()
        torch.cuda.synchronize()
        if k >= args.warmup:
            times.append(time.perf_counter() - t0)
            dev_t.append(e0.elapsed_time(e1) / 1e3)
    t_batch = statistics.mean(times)
    sample = mols[:24]
    loop_t = []
    for rep in range(2):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        E_loop = []
        for mol in sample:
            E_loop.append(rhf(GpuEngine(mol).prepare()).E)
        torch.cuda.synchronize()
        loop_t.append(time.perf_counter() - t0)
    per = min(loop_t) / len(sample)
    dE = max(abs(a - b) for a, b in zip(E_loop, res.E[:len(sample)]))
    return {"workload": "1024 instances cycling H2O, NH3, CH4, HF, CH3OH, C2H6, 6-31G, N(0, 0.08 A) jitter",
            "instances": n, "batched_s": t_batch, "batched_device_s": statistics.mean(dev_t),
            "instances_per_s": n / t_batch, "looped_instances_per_s": 1.0 / per, "speedup_vs_loop": per * n / t_batch,
            "converged": int(res.converged.sum()), "mean_scf_iterations": float(res.iterations.mean()),
            "max_scf_iterations": int(res.iterations.max()), "quartets": eng.stats["quartets"],
            "max_dE_vs_loop": dE, "loop_sample": "first %d instances, one GpuEngine + rhf each" % len(sample)}


def learned_leg(torch, args, n=1024):
    """Held-out generated molecules (<= 6 heavy atoms from C/N/O plus H, N(0, 0.1 A)
    jitter, seed 2, never seen in training), 6-31G, one batch: plain FP64 batched SCF
    from the SAD guess against the learned-guess, mixed-precision batched SCF (quartets
    with Schwarz bound below 1e-4 in FP32; dense steps in FP32 until the DIIS residual
    RMS is below 1e-4), and against looping the plain FP64 one-molecule GPU SCF.  Timed
    from Molecule objects to converged energies."""
    import numpy as np
    from pychem_gb300.engine import GpuEngine
    from pychem_gb300.ensemble import EnsembleEngine, rhf_batched
    from pychem_gb300.learned.mlp import PairMLP
    from pychem_gb300.learned.molgen import molecules
    from pychem_gb300.learned.train import WEIGHTS, guess_density
    from pychem_gb300.molecule import Molecule
    from pychem_gb300.scf import rhf
    if not os.path.exists(WEIGHTS):
        return {"unavailable": "no trained weights"}
    net = PairMLP.load(WEIGHTS)
    mols = [Molecule(c, "6-31G") for c in molecules(n, seed=2)]

    def plain():
        eng = EnsembleEngine(mols).prepare()
        return eng, rhf_batched(eng, guess="sad")

    def learned():
        eng = EnsembleEngine(mols, precision="mixed", fp32_below=1e-4).prepare()
        return eng, rhf_batched(eng, D0=guess_density(net, mols, eng), dense_fp32_until=1e-4)

    out = {"workload": "%d held-out generated molecules (<= 6 heavy atoms C/N/O + H), 6-31G, up to %d AO"
                       % (n, max(m.NOrbitals for m in mols))}
    res = {}
    for name, fn in (("plain_fp64_sad", plain), ("learned_mixed", learned)):
        ts = []
        for k in range(1 + max(1, min(args.steps, 2))):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            eng, r = fn()
            torch.cuda.synchronize()
            if k >= 1:
                ts.append(time.perf_counter() - t0)
            del eng
        res[name] = r
        out[name] = {"ttc_s": statistics.mean(ts), "instances_per_s": n / statistics.mean(ts),
                     "mean_scf_iterations": float(r.iterations.mean()), "max_scf_iterations": int(r.iterations.max()),
                     "converged": int(r.converged.sum())}
    dE = res["learned_mixed"].E - res["plain_fp64_sad"].E
    out["max_abs_dE_learned_mixed_vs_plain"] = float(np.abs(dE).max())
    out["ttc_ratio_plain_over_learned_mixed"] = out["plain_fp64_sad"]["ttc_s"] / out["learned_mixed"]["ttc_s"]
    sample = mols[:16]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    E_loop = [rhf(GpuEngine(m).prepare()).E for m in sample]
    torch.cuda.synchronize()
    per = (time.perf_counter() - t0) / len(sample)
    out["looped_plain_fp64_instances_per_s"] = 1.0 / per
    out["ttc_ratio_looped_plain_over_learned_mixed"] = per * n / out["learned_mixed"]["ttc_s"]
    out["max_abs_dE_loop_vs_learned_mixed"] = float(max(abs(a - b) for a, b in zip(E_loop, res["learned_mixed"].E)))
    return out


def alkane_leg(torch, args):
    """C12H26 / cc-pVDZ (298 AO, s/p/d): plain FP64 vs mixed precision (quartets with
    Schwarz bound below 1e-4 in FP32, everything else and all accumulation in FP64)."""
    from pychem_gb300 import workloads as W
    from pychem_gb300.engine import GpuEngine
    from pychem_gb300.molecule import Molecule
    from pychem_gb300.scf import rhf
    mol = Molecule(W.alkane(12, seed=SEED), "cc-pVDZ")
    out = {"workload": "C12H26 all-trans, N(0, 0.03 A) jitter, cc-pVDZ, %d AO" % mol.NOrbitals}
    for prec in ("fp64", "mixed"):
        eng = GpuEngine(mol, precision=prec, fp32_below=1e-4)
        ts, te = [], []
        for k in range(2 + max(1, min(args.steps, 2))):
            torch.cuda.synchronize()
            e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
            e0.record()
            eng.compute_pair_data(); eng.one_electron(); eng.schwarz(); eng.build_tasks()
            e1.record()
            eng.compute_eris()
            e2.record()
            r = rhf(eng)
            torch.cuda.synchronize()
            if k >= 2:
                te.append(e1.elapsed_time(e2) / 1e3)
                ts.append(e0.elapsed_time(e1) / 1e3)
            t_tot = None
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        eng.compute_pair_data(); eng.one_electron(); eng.schwarz(); eng.build_tasks(); eng.compute_eris()
        r = rhf(eng)
        torch.cuda.synchronize()
        out[prec] = {"ttc_s": time.perf_counter() - t0, "eri_s": statistics.mean(te), "E_rhf": r.E,
                     "iterations": r.iterations, "quartets_fp32": eng.stats["quartets_fp32"],
                     "quartets_fp64": eng.stats["quartets_fp64"]}
    out["dE_mixed_vs_fp64"] = out["mixed"]["E_rhf"] - out["fp64"]["E_rhf"]
    ref = oracle_energies().get("c3_c12h26_ccpvdz")
    if ref:
        out["E_rhf_oracle"] = ref["E_rhf"]
        out["dE_fp64_vs_oracle"] = out["fp64"]["E_rhf"] - ref["E_rhf"]
        out["dE_mixed_vs_oracle"] = out["mixed"]["E_rhf"] - ref["E_rhf"]
    out["eri_speedup_mixed"] = out["fp64"]["eri_s"] / out["mixed"]["eri_s"]
    return out


def noci_leg(torch, args):
    """Spin-flip NOCI (Methods/noci.py) on C2 (r = 1.25 A) / cc-pVDZ with SFD-CISD
    determinants: the state SCFs in the reference's order (high spin first), the
    spin-flip determinants, the CI matrix over every determinant pair (J/K of all
    co-densities in one batched digestion per integral class) and the generalised
    eigenproblem.  cpu_noci_matrix_s: the oracle's CI matrix (numpy, dense ERI einsums,
    one core) on a bounded sample of the same pairs, extrapolated to all of them."""
    import numpy as np
    from pychem_gb300 import noci
    from pychem_gb300.engine import GpuEngine
    from pychem_gb300.molecule import Molecule
    from oracle import oracle
    mol = Molecule([["C", 6.0, 0.0, 0.0, 0.0], ["C", 6.0, 1.25, 0.0, 0.0]], "cc-pVDZ")
    exc = "SFD-CISD"
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    eng = GpuEngine(mol).prepare()
    out = noci.run(eng, exc, reference="UHF", constrain_excited=True)
    torch.cuda.synchronize()
    t_total = time.perf_counter() - t0
    na, nb = mol.NAlphaElectrons, mol.NBetaElectrons
    da, db = out["dets_alpha"], out["dets_beta"]
    m = len(da)
    ts = []
    for _ in range(3):
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        Hci, Sci = noci.noci_matrix(eng, da, db, na, nb)
        noci.generalized_eigh(Hci, Sci)
        b.record()
        torch.cuda.synchronize()
        ts.append(a.elapsed_time(b) / 1e3)
    t_ci = min(ts)
    npairs = m * (m + 1) // 2
    # CPU: the oracle on a bounded sample of pairs
    S, H = eng.S.cpu().numpy(), eng.H.cpu().numpy()
    eri = eng.dense_eri().cpu().numpy()
    e_nuc = mol.nuclear_repulsion()
    Da = [x.cpu().numpy() for x in da]
    Db = [x.cpu().numpy() for x in db]
    pairs = [(i, j) for i in range(m) for j in range(i + 1)]
    rng = np.random.default_rng(SEED)
    sample = [pairs[k] for k in rng.choice(len(pairs), size=min(24, len(pairs)), replace=False)]
    c0 = time.perf_counter()
    for i, j in sample:
        oracle.noci_element(Da[i], Db[i], Da[j], Db[j], S, H, eri, na, nb, e_nuc)
    cpu_per_pair = (time.perf_counter() - c0) / len(sample)
    e = out["energies"].cpu().numpy()
    return {"workload": "C2 r=1.25 A, cc-pVDZ (%d AO), %s: %d determinants, %d pairs" % (eng.nbf, exc, m, npairs),
            "ttc_s": t_total, "ci_matrix_and_eigh_s": t_ci, "pairs_per_s": npairs / t_ci,
            "hf_state_energies": [r.E for r in out["hf"]], "hf_iterations": [r.iterations for r in out["hf"]],
            "noci_lowest": [float(x) for x in e[:3]],
            "cpu_noci_matrix_s": cpu_per_pair * npairs, "cpu_sample_pairs": len(sample), "cpu_cores": 1,
            "ci_speedup_vs_cpu_oracle": cpu_per_pair * npairs / t_ci}


def _cpu_scat_worker(args):
    """Time the C oracle on a list of j0(S r12) quartets (one process, operator set)."""
    atoms, basis, S, quads = args
    import ctypes
    import numpy as np
    from oracle import oracle as O
    b = O.Basis(atoms, basis)
    O.lib().oracle_set_operator(1, float(S))
    q = np.ascontiguousarray(np.asarray(quads, dtype=np.int32).reshape(-1))
    t0 = time.perf_counter()
    O.lib().oracle_eri_list(b.c, len(quads), q.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
    t = time.perf_counter() - t0
    O.lib().oracle_set_operator(0, 0.0)
    return t


def scattering_leg(torch, args):
    """Total electron-scattering intensities (Methods/properties.py) of the RHF ground
    state of (H2O)8 / 6-31G on a 16-point grid S = 0 .. 7.5 bohr^-1: per grid value the
    j0(S r12) Schwarz pass, quartet plan, integral store and contraction with the
    state's densities.  CPU: the C oracle's j0(S r12) quartets/s on a bounded sample
    at S = 2, times the quartets its screen keeps there (contraction not added)."""
    import numpy as np
    from pychem_gb300 import scattering, workloads as W
    from pychem_gb300.engine import GpuEngine
    from pychem_gb300.molecule import Molecule
    from pychem_gb300.scf import rhf
    from oracle import oracle as O
    mol = Molecule(W.water_cluster(2, 2, 2, seed=SEED), "6-31G")
    r = rhf(GpuEngine(mol).prepare())
    grid = [0.5 * k for k in range(16)]
    dens = [(r.D, r.D)]
    scattering.intensities(mol, grid[:2], dens)            # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    table = scattering.intensities(mol, grid, dens)
    torch.cuda.synchronize()
    t_gpu = time.perf_counter() - t0
    # CPU sample at S = 2
    atoms = [(a[0], a[1], *a[2]) for a in mol.atoms]
    b = O.Basis(atoms, "6-31G")
    S_cpu = 2.0
    O.lib().oracle_set_operator(1, S_cpu)
    try:
        quads = np.array(b.quartets(), dtype=np.int32)
    finally:
        O.lib().oracle_set_operator(0, 0.0)
    rng = np.random.default_rng(SEED)
    probe = quads[rng.choice(len(quads), size=min(len(quads), 1500), replace=False)]
    per = _cpu_scat_worker((atoms, "6-31G", S_cpu, probe)) / len(probe)
    n = int(min(len(quads), max(1500, 10.0 / per)))
    sample = quads[rng.choice(len(quads), size=n, replace=False)]
    rate = n / _cpu_scat_worker((atoms, "6-31G", S_cpu, sample))
    return {"workload": "(H2O)8 6-31G (%d AO), RHF ground state, %d grid values S = 0..%.1f" % (
                mol.NOrbitals, len(grid), grid[-1]),
            "gpu_s": t_gpu, "gpu_s_per_grid_value": t_gpu / len(grid),
            "intensity_S0": float(table[0, 0]), "intensity_S2": float(table[4, 0]),
            "cpu_quartets_per_s": rate, "cpu_quartets_S2": int(len(quads)),
            "cpu_s_per_grid_value_S2": len(quads) / rate, "cpu_sample": "%d of %d quartets at S = 2, 1 core" % (
                n, len(quads)),
            "speedup_per_grid_value": (len(quads) / rate) / (t_gpu / len(grid))}


def gpu_arm(args):
    import numpy as np
    import torch
    rank, world, local = env_rank()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from pychem_gb300 import _lib, workloads as W
    from pychem_gb300.api import rhf_mp2
    from pychem_gb300.engine import GpuEngine
    from pychem_gb300.molecule import Molecule
    from pychem_gb300.scf import mp2_flops, rhf, rmp2

    coords = W.water_cluster(seed=SEED)
    mol = Molecule(coords, "6-31G")
    n, o = mol.NOrbitals, mol.NAlphaElectrons
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")   # 256 MiB > 129 MB L2

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    def solve(eng):
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(5)]
        ev[0].record()
        eng.compute_pair_data()
        eng.one_electron(); eng.schwarz(); eng.build_tasks()
        ev[1].record()
        eng.compute_eris()
        ev[2].record()
        # MP2's pair tensor (from the ERI store alone) is built on a side stream beside the SCF
        eri, ready = eng.prefetch_mp2_tensor()
        r = rhf(eng)
        ev[3].record()
        torch.cuda.current_stream().wait_event(ready)
        e2 = rmp2(eng, r.C, r.eps, eri=eri)
        del eri
        ev[4].record()
        return r, e2, ev

    def run(precision, k_steps, warm):
        eng = GpuEngine(mol, precision=precision)
        for _ in range(warm):
            solve(eng)
        times, phases, res = [], [], None
        launches0 = _lib.launch_count
        for _ in range(k_steps):
            flush.zero_()
            barrier()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            r, e2, ev = solve(eng)
            e1.record()
            barrier()
            times.append(e0.elapsed_time(e1) / 1e3)
            phases.append([ev[i].elapsed_time(ev[i + 1]) / 1e3 for i in range(4)])
            res = (r, e2)
        launches = (_lib.launch_count - launches0) / max(1, k_steps)
        return eng, times, phases, res, launches

    peaks = load_peaks()
    fp64_peak = probe_peak(torch, _lib, False)
    fp32_peak = probe_peak(torch, _lib, True)

    with Clocks(local) as clk:
        eng, times, phases, (r, e2), launches = run("fp64", args.steps, args.warmup)
    clocks = clk.summary()
    # mixed precision: same solve, quartets below the 1e-4 Schwarz bound in FP32
    engm, times_m, phases_m, (rm, e2m), _ = run("mixed", max(1, args.steps), 1)

    t_step = statistics.mean(times)
    ph = [statistics.mean(p[i] for p in phases) for i in range(4)]
    ops = {s["cls"]: s for s in json.load(open(os.path.join(REPO, "pychem_gb300", "csrc", "eri_ops.json")))}
    names = list(ops)
    eri_flops = 0.0
    for (cls, part), npq in eng.prim_quartets.items():
        st = ops[names[cls]]
        nq = eng.classes[cls][part][1]
        eri_flops += float(npq) * (st["vrr_flops"] + st["overhead_flops"]) + nq * st["finish_flops"]
    quartets = eng.stats["quartets"]
    # Fock builds in isolation (digestion + symmetrisation)
    D = r.D.contiguous()
    fk = []
    for _ in range(5):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(); eng.fock(D); b.record(); torch.cuda.synchronize()
        fk.append(a.elapsed_time(b) / 1e3)
    t_fock = min(fk)
    # ERI pass alone (for the roofline of the dominant kernels)
    eri_t = []
    for _ in range(3):
        flush.zero_()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(); eng.compute_eris(); b.record(); torch.cuda.synchronize()
        eri_t.append(a.elapsed_time(b) / 1e3)
    t_eri = min(eri_t)
    store_bytes = sum(s.numel() * 8 for s in eng.stores.values())

    # end to end through the public API with host buffers
    e2e_t = []
    for k in range(max(1, args.steps)):
        flush.zero_()
        barrier()
        t0 = time.perf_counter()
        out = rhf_mp2(coords, "6-31G")
        torch.cuda.synchronize()
        e2e_t.append(time.perf_counter() - t0)
    t_e2e = statistics.mean(e2e_t)
    # the dominant kernel: the four tensor-core Ozaki launches of the MP2 transform,
    # timed one by one on the launching stream; algorithmic work = the BF16 tensor
    # flops of the digit-slice products, 2 M N Kp per product, 21 products (6 slices,
    # levels up to 7), Kp = K rounded up to the 32-column chunk
    from pychem_gb300.scf import mp2_transform, ozaki_tc_status
    Ep = eng.dense_eri_pairs(compact=True)
    tc_t, tc_flops = 0.0, 0.0
    tc_runs = []
    for _ in range(3):
        flush.zero_()
        torch.cuda.synchronize()
        tl = []
        mp2_transform(Ep, r.C[:, :o].contiguous(), r.C[:, o:].contiguous(), timings=tl)
        torch.cuda.synchronize()
        tc_runs.append(tl)
    tl = tc_runs[-1]
    for (M_, N_, K_, ev) in tl:
        kp = (K_ + 31) // 32 * 32
        ncols = (N_ + 63) // 64 * 64 if N_ > 80 else N_
        tc_flops += 21 * 2.0 * M_ * ncols * kp
        tc_t += ev[0].elapsed_time(ev[1]) / 1e3
    tc_status = ozaki_tc_status("cuda")
    tc_bytes = sum(M_ * K_ * 8 + M_ * N_ * 8 for (M_, N_, K_, _) in tl)
    del Ep
    # cross-check of the tensor-core MP2 transform against cuBLAS DGEMM (untimed)
    e2_fp64 = rmp2(eng, r.C, r.eps, gemm="fp64")
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(); rmp2(eng, r.C, r.eps, gemm="fp64"); b.record(); torch.cuda.synchronize()
    t_mp2_fp64 = a.elapsed_time(b) / 1e3

    ens = ensemble_leg(torch, args) if world == 1 or rank == 0 else None
    alk = alkane_leg(torch, args) if world == 1 or rank == 0 else None
    lrn = learned_leg(torch, args) if world == 1 or rank == 0 else None
    nci = noci_leg(torch, args) if world == 1 or rank == 0 else None
    sct = scattering_leg(torch, args) if world == 1 or rank == 0 else None

    # max over ranks
    if world > 1:
        tt = torch.tensor([t_step, t_e2e], device="cuda")
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        t_step, t_e2e = float(tt[0]), float(tt[1])
    if rank != 0:
        return

    cpu = None
    if world == 1:
        atoms_b = [(a[0], a[1], *a[2]) for a in mol.atoms]
        ref_c2 = oracle_energies().get("c2_water16_631g", {})
        cores = os.cpu_count() or 1
        v_cpu, desc, parts = cpu_full_estimate(atoms_b, "6-31G", o, int(ref_c2.get("scf_iterations", 31)), cores,
                                               target_s=3.0)
        cpu = {"value": v_cpu, "unit": "s", "cores": cores, "kind": "port", "sample": desc, "breakdown_s": parts}

    achieved = eri_flops / t_eri / 1e12
    ref = oracle_energies().get("c2_water16_631g", {})
    vs_oracle = {"E_rhf_oracle": ref.get("E_rhf"), "E_mp2_corr_oracle": ref.get("E_mp2_corr"),
                 "dE_rhf": r.E - ref["E_rhf"] if ref else None,
                 "dE_mp2_corr": e2 - ref["E_mp2_corr"] if ref else None,
                 "dE_rhf_mixed": rm.E - ref["E_rhf"] if ref else None,
                 "dE_mp2_corr_mixed": e2m - ref["E_mp2_corr"] if ref else None}
    line = {
        "metric": METRIC, "value": t_step, "unit": "s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "basis": "6-31G", "nbf": n, "n_occ": o, "seed": SEED,
                   "screening": "Schwarz 1e-8", "scf": "|dE|<1e-10 and D-RMS<1e-8, DIIS(10)",
                   "l2": "256 MiB buffer written between steps", "parallelism": "replicas" if world > 1 else "single"},
        "E_rhf": r.E, "E_mp2_total": r.E + e2, "scf_iterations": r.iterations, "vs_oracle": vs_oracle,
        "eri_shell_quartets": quartets,
        "eri_quartets_per_s": quartets / t_eri,
        "fock_builds_per_s": 1.0 / t_fock,
        "mp2_tflops": mp2_flops(n, o, n - o) / ph[3] / 1e12,
        "mp2": {"gemm": "tcgen05 BF16 tensor cores, Ozaki digit slices (6), all levels in one kernel (pcg_ozaki_gemm_tc)",
                "s": ph[3], "tc_launches_s": tc_t, "tc_error_flag": tc_status,
                "dE_vs_fp64_dgemm": e2 - e2_fp64, "fp64_dgemm_s": t_mp2_fp64,
                "fp64_dgemm_tflops": mp2_flops(n, o, n - o) / t_mp2_fp64 / 1e12},
        "phases_s": {"setup_1e_schwarz_tasks": ph[0], "eri": ph[1], "scf": ph[2], "mp2": ph[3],
                     "note": "MP2's compact pair tensor is built on a side stream during the SCF phase"},
        "mixed": {"value": statistics.mean(times_m), "unit": "s", "fp32_below": 1e-4,
                  "quartets_fp32": engm.stats["quartets_fp32"], "quartets_fp64": engm.stats["quartets_fp64"],
                  "dE_rhf_vs_fp64": rm.E - r.E, "dE_mp2_vs_fp64": (rm.E + e2m) - (r.E + e2),
                  "eri_s": statistics.mean(p[1] for p in phases_m)},
        "roofline": {"bound": "tensor", "kernel": "k_ozt_gemm (tcgen05 Ozaki GEMM, the four MP2 quarter transforms)",
                     "achieved": tc_flops / tc_t / 1e12, "peak": peaks.get("bf16_tflops"), "unit": "TFLOP/s",
                     "frac": (tc_flops / tc_t / 1e12) / peaks["bf16_tflops"] if peaks.get("bf16_tflops") else None,
                     "peak_source": "MEASURED_PEAKS.json bf16_tflops (burst), of measured",
                     "traffic": tc_bytes / max(1, len(tl)),
                     "traffic_source": "ncu capture of one launch at the first transform's shape "
                                       "(profiles/ozaki_tc_gemm_mp2_shape.md): DRAM reads = the FP64 input "
                                       "once, writes = the FP64 output; scaled to each launch's M, N, K and "
                                       "averaged per launch",
                     "algorithmic_flops_per_launch": tc_flops / max(1, len(tl)),
                     "launches": len(tl), "seconds": tc_t,
                     "fp64_operand_and_output_bytes": tc_bytes},
        "roofline_eri": {"bound": "fp64", "kernel": "ERI class kernels k_eri<*> (FP64 pipe)",
                         "achieved": achieved, "peak": fp64_peak, "unit": "TFLOP/s", "frac": achieved / fp64_peak,
                         "peak_source": "measured by bench.py FP64 FMA probe (pcg_fma_probe); MEASURED_PEAKS.json has no FP64 figure",
                         "traffic": None, "algorithmic_flops": eri_flops, "eri_pass_s": t_eri},
        "peaks": {"fp64_tflops_probe": fp64_peak, "fp32_tflops_probe": fp32_peak,
                  "hbm_gbs": peaks.get("hbm_gbs"), "bf16_tflops": peaks.get("bf16_tflops")},
        "fock_digest": {"s_per_build": t_fock, "store_bytes": store_bytes,
                        "hbm_frac": store_bytes / t_fock / 1e9 / peaks["hbm_gbs"] if peaks.get("hbm_gbs") else None},
        "cpu_baseline": cpu,
        "ensemble": ens,
        "alkane_mixed": alk,
        "learned_guess": lrn,
        "noci_spin_flip": nci,
        "scattering": sct,
        "e2e": {"value": t_e2e, "unit": "s", "h2d_bytes_per_step": out["h2d_bytes"],
                "d2h_bytes_per_step": out["d2h_bytes"]},
        "gpu_launches": launches,
        "clocks": clocks,
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    args = ap.parse_args()
    if args.impl == "reference":
        reference_arm(args)
    else:
        gpu_arm(args)


if __name__ == "__main__":
    main()
