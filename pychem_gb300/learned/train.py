"""Train and evaluate the learned initial guess on the GPU.

    python -m pychem_gb300.learned.train [--n-train 50000] [--n-test 2000] [--epochs 8]

1. training molecules (molgen, seed 1) and held-out molecules (seed 2), 6-31G;
2. converged RHF densities of the training molecules from the batched SCF
   (EnsembleEngine + rhf_batched, SAD guess), in chunks of similar size;
3. pair features and bond-frame block targets (blocks.py), normalised per slot;
4. Adam on the masked squared error with the library's forward/backward kernels;
5. held-out evaluation: batched SCF from the SAD guess and from the learned guess,
   SCF iterations, time-to-convergence and |dE| between the two;
6. weights and the report are written to pychem_gb300/data/learned_guess_631g.{npz,json}.
"""
import argparse
import json
import os
import time

import numpy as np
import torch

from ..ensemble import EnsembleEngine, rhf_batched, sad_batch
from ..molecule import Molecule
from . import blocks as B
from .mlp import PairMLP
from .molgen import molecules

HERE = os.path.dirname(os.path.abspath(__file__))
DATA = os.path.join(os.path.dirname(HERE), "data")
WEIGHTS = os.path.join(DATA, "learned_guess_631g.npz")
REPORT = os.path.join(DATA, "learned_guess_631g.json")
BASIS = "6-31G"


def chunks_by_size(mols, max_batch=1024, quartet_budget=1.5e8):
    order = np.argsort([m.NOrbitals for m in mols], kind="stable")
    out, cur, q = [], [], 0.0
    for i in order:
        ns = mols[i].NCgtf
        qi = (ns * (ns + 1) / 2) ** 2 / 2
        if cur and (len(cur) >= max_batch or q + qi > quartet_budget):
            out.append(cur)
            cur, q = [], 0.0
        cur.append(int(i))
        q += qi
    if cur:
        out.append(cur)
    return out


def solve(mols, D0=None, guess="sad"):
    eng = EnsembleEngine(mols).prepare()
    res = rhf_batched(eng, guess=guess, D0=D0)
    return eng, res


TYPE_LIST = list(B.TYPES)


def _block_index(mol, r0, c0, ni, nj, n):
    """Flat indices into a (B, n, n) tensor of the (ni x nj) blocks at (r0, c0)."""
    dev = mol.device
    ri = torch.arange(ni, device=dev)[None, :, None]
    cj = torch.arange(nj, device=dev)[None, None, :]
    return ((mol[:, None, None] * n + r0[:, None, None] + ri) * n + c0[:, None, None] + cj).reshape(-1)


def assemble(D, pc, par):
    """Add predicted blocks to D (B, n, n): off-diagonal slots averaged over the two
    orders of a pair, diagonal corrections summed over neighbours (atomic adds)."""
    n = D.shape[-1]
    flat = D.view(-1)
    R = B.frames(pc["vec"].to(torch.float64))
    par = par.to(torch.float64)
    for c, (ti, tj) in enumerate(TYPE_LIST):
        sel = (pc["tc"] == c).nonzero().squeeze(1)
        if sel.numel() == 0:
            continue
        ni, nj = B.nao_of(ti), B.nao_of(tj)
        m, ai, aj = pc["mol"][sel], pc["ao_i"][sel], pc["ao_j"][sel]
        blk = 0.5 * B.blocks_from_params(par[sel, :B.NOFF], R[sel], ti, tj)
        flat.index_add_(0, _block_index(m, ai, aj, ni, nj, n), blk.reshape(-1))
        flat.index_add_(0, _block_index(m, aj, ai, nj, ni, n), blk.transpose(1, 2).reshape(-1))
        dg = B.diag_from_params(par[sel, B.NOFF:], R[sel], ti)
        flat.index_add_(0, _block_index(m, ai, ai, ni, ni, n), dg.reshape(-1))
    return D


def guess_density(net, mols, eng=None, device="cuda"):
    """SAD plus the network's pair blocks and diagonal corrections, (B, nmax, nmax),
    scaled to the electron count when the engine's overlap is available."""
    if eng is None:
        eng = EnsembleEngine(mols)
    D = sad_batch(eng)
    pc = B.pairs(eng.atom_table(), D.device)
    par = net.predict(B.features(pc, D.device))
    D = assemble(D, pc, par)
    # rescale to the molecule's electron count: tr(D S) = N_alpha
    S = getattr(eng, "S", None)
    if S is not None:
        ne = torch.tensor([m.NAlphaElectrons for m in mols], dtype=torch.float64, device=D.device)
        D *= (ne / torch.einsum("bij,bji->b", D, S))[:, None, None]
    return D


def build_dataset(mols_all, chunks, device="cuda", seed=0):
    """Pairs (features, off-diagonal slot targets, frames, atom index) and atoms (change
    of the converged diagonal block from the free-atom block) of every converged
    molecule, molecules in a seeded random order so that contiguous ranges are batches."""
    P, A = [], []
    nmol = natom = 0
    for idx in chunks:
        mols = [mols_all[i] for i in idx]
        eng, res = solve(mols)
        Dc = res.D
        dev = Dc.device
        Ds = sad_batch(eng)
        at = eng.atom_table()
        pc = B.pairs(at, dev)
        conv = torch.as_tensor(res.converged, device=dev)
        # converged diagonal blocks minus the free-atom blocks, 9x9 padded
        r9 = torch.arange(9, device=dev)
        am = torch.as_tensor(at["mol"], device=dev)[:, None, None]
        a0 = torch.as_tensor(at["ao0"], device=dev)[:, None, None]
        isH = torch.as_tensor(at["z"] == 1.0, device=dev)
        lim = torch.where(isH, 2, 9)[:, None, None]
        ii = (a0 + r9[None, :, None]).clamp_max(Dc.shape[1] - 1)
        jj = (a0 + r9[None, None, :]).clamp_max(Dc.shape[1] - 1)
        valid = (r9[None, :, None] < lim) & (r9[None, None, :] < lim)
        dD = torch.where(valid, Dc[am, ii, jj] - Ds[am, ii, jj], 0.0).to(torch.float32)
        # off-diagonal targets
        tc = pc["tc"]
        T = torch.zeros(tc.numel(), B.NOFF, dtype=torch.float64, device=dev)
        Mk = torch.zeros(tc.numel(), B.NOFF, dtype=torch.float32, device=dev)
        R = B.frames(pc["vec"])
        for c, t in enumerate(TYPE_LIST):
            sel = (tc == c).nonzero().squeeze(1)
            if sel.numel() == 0:
                continue
            blk = B.gather_blocks(Dc, {k: pc[k][sel] for k in ("mol", "ao_i", "ao_j")}, t)
            par, mask = B.params_from_blocks(blk, R[sel], *t)
            T[sel] = par
            Mk[sel] = mask.to(torch.float32)
        kp = conv[pc["mol"]].nonzero().squeeze(1)
        ka = conv[am[:, 0, 0]].nonzero().squeeze(1)
        # molecules (converged ones) and atoms renumbered over all chunks
        newid = torch.cumsum(conv.to(torch.int64), 0) - 1 + nmol
        aidx = torch.cumsum(conv[am[:, 0, 0]].to(torch.int64), 0) - 1 + natom
        P.append(dict(X=B.features({k: v[kp] for k, v in pc.items()}, dev), T=T[kp].to(torch.float32), M=Mk[kp],
                      R=R[kp].to(torch.float32), tc=tc[kp], gi=aidx[pc["gi"][kp]], mol=newid[pc["mol"][kp]]))
        A.append(dict(dD=dD[ka], isH=isH[ka], mol=newid[am[ka, 0, 0]]))
        nmol += int(conv.sum())
        natom += ka.numel()
        del eng, res, Dc, Ds
        torch.cuda.empty_cache()
    pairs = {k: torch.cat([x[k] for x in P]) for k in P[0]}
    atoms = {k: torch.cat([x[k] for x in A]) for k in A[0]}
    # seeded random molecule order; atoms and pairs re-sorted to it
    dev = pairs["X"].device
    perm = torch.as_tensor(np.random.default_rng(seed).permutation(nmol), device=dev)
    ao = torch.argsort(perm[atoms["mol"]], stable=True)
    inv = torch.empty_like(ao)
    inv[ao] = torch.arange(ao.numel(), device=dev)
    po = torch.argsort(perm[pairs["mol"]], stable=True)
    pairs = {k: v[po] for k, v in pairs.items()}
    pairs["gi"] = inv[pairs["gi"]]
    pairs["mol"] = perm[pairs["mol"]].cpu().numpy()
    atoms = {k: v[ao] for k, v in atoms.items()}
    atoms["mol"] = perm[atoms["mol"]].cpu().numpy()
    return pairs, atoms, nmol


def _diag_loss(Yd, R, tc, gi_local, dD, nent, dscale):
    """Squared error of the summed diagonal corrections against the converged change,
    in units of dscale; returns (loss, dL/dYd)."""
    Yd = Yd.detach().requires_grad_(True)
    pred = torch.zeros_like(dD)
    for c, (ti, _) in enumerate(TYPE_LIST):
        sel = (tc == c).nonzero().squeeze(1)
        if sel.numel() == 0:
            continue
        blk = B.diag_from_params(Yd[sel] * dscale, R[sel], ti)
        ni = blk.shape[1]
        blk = torch.nn.functional.pad(blk, (0, 9 - ni, 0, 9 - ni))
        pred = pred.index_add(0, gi_local[sel], blk)
    loss = ((pred - dD) ** 2).sum() / (nent * dscale * dscale)
    loss.backward()
    return loss.detach(), Yd.grad


def train(pairs, atoms, nmol, epochs=8, mols_per_batch=96, lr=1e-3, seed=0, log=None):
    X, T, M = pairs["X"], pairs["T"], pairs["M"]
    dev = X.device
    net = PairMLP(seed=seed, device=dev)
    cnt = M.sum(0).clamp_min(1.0)
    mean = (T * M).sum(0) / cnt
    var = (((T - mean) * M) ** 2).sum(0) / cnt
    std = var.sqrt().clamp_min(1e-6)
    dD = atoms["dD"]
    nent_all = torch.where(atoms["isH"], 4, 81).sum()
    dscale = float((dD.pow(2).sum() / nent_all).sqrt())
    net.mean = torch.cat([mean, torch.zeros(B.NDIAG, device=dev)])
    net.std = torch.cat([std, torch.full((B.NDIAG,), dscale, device=dev)])
    zpad = torch.zeros(X.shape[0], B.NDIAG, device=dev)
    Tn = torch.cat([((T - mean) / std) * M, zpad], 1)
    Mf = torch.cat([M, zpad], 1)
    pm, am = pairs["mol"], atoms["mol"]
    bounds = np.arange(0, nmol + mols_per_batch, mols_per_batch)
    pb = np.searchsorted(pm, bounds)
    ab = np.searchsorted(am, bounds)
    nb = len(bounds) - 1
    rng = np.random.default_rng(seed)
    steps = epochs * nb
    step = 0
    hist = []
    for ep in range(epochs):
        tot_o = tot_d = 0.0
        for b in rng.permutation(nb):
            p0, p1, a0, a1 = pb[b], pb[b + 1], ab[b], ab[b + 1]
            if p1 <= p0:
                continue
            Y, cache = net.forward(X[p0:p1], keep=True)
            lo, dY = net.loss_grad(Y, Tn[p0:p1], Mf[p0:p1])
            nent = torch.where(atoms["isH"][a0:a1], 4, 81).sum()
            ld, gd = _diag_loss(Y[:, B.NOFF:], pairs["R"][p0:p1], pairs["tc"][p0:p1], pairs["gi"][p0:p1] - a0,
                                dD[a0:a1], nent, dscale)
            dY[:, B.NOFF:] += gd
            grads = net.backward(dY, cache)
            frac = step / max(steps - 1, 1)
            net.adam(grads, lr * (0.05 + 0.95 * 0.5 * (1 + np.cos(np.pi * frac))))
            tot_o += float(lo)
            tot_d += float(ld)
            step += 1
        hist.append([tot_o / nb, tot_d / nb])
        if log:
            log("epoch %d loss off-diagonal %.5f diagonal %.5f" % (ep, tot_o / nb, tot_d / nb))
    return net, hist


def evaluate(net, test_mols, chunks):
    out = {"sad_iterations": [], "learned_iterations": [], "dE": [], "sad_s": 0.0, "learned_s": 0.0,
           "fallbacks": 0, "n": 0}
    for idx in chunks:
        mols = [test_mols[i] for i in idx]
        eng = EnsembleEngine(mols).prepare()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r_sad = rhf_batched(eng, guess="sad")
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        D0 = guess_density(net, mols, eng)
        r_nn = rhf_batched(eng, D0=D0)
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        Ds = sad_batch(eng)
        for key, G in (("sad_err", Ds), ("learned_err", D0)):
            out.setdefault(key, []).extend(torch.sqrt(torch.mean((G - r_sad.D) ** 2, dim=(1, 2))).tolist())
        ne = torch.tensor([m.NElectrons for m in mols], dtype=torch.float64, device=D0.device)
        out.setdefault("learned_dN", []).extend((2.0 * torch.einsum("bij,bji->b", D0, eng.S) - ne).tolist())
        bad = ~r_nn.converged
        out["fallbacks"] += int(bad.sum())
        E_nn = np.where(bad, r_sad.E, r_nn.E)
        out["sad_iterations"] += [int(x) for x in r_sad.iterations]
        out["learned_iterations"] += [int(x) for x in np.where(bad, r_sad.iterations, r_nn.iterations)]
        out["dE"] += [float(x) for x in (E_nn - r_sad.E)]
        out["sad_s"] += t1 - t0
        out["learned_s"] += t2 - t1
        out["n"] += len(mols)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n-train", type=int, default=50000)
    ap.add_argument("--n-test", type=int, default=2000)
    ap.add_argument("--epochs", type=int, default=8)
    ap.add_argument("--out", default=WEIGHTS)
    args = ap.parse_args()
    t_start = time.time()
    log = lambda s: print("[%.0fs] %s" % (time.time() - t_start, s), flush=True)
    train_coords = molecules(args.n_train, seed=1)
    test_coords = molecules(args.n_test, seed=2)
    train_mols = [Molecule(c, BASIS) for c in train_coords]
    test_mols = [Molecule(c, BASIS) for c in test_coords]
    log("molecules built")
    pairs, atoms, nconv = build_dataset(train_mols, chunks_by_size(train_mols))
    log("dataset: %d pairs, %d atoms from %d converged SCFs" % (pairs["X"].shape[0], atoms["dD"].shape[0], nconv))
    net, hist = train(pairs, atoms, nconv, epochs=args.epochs, log=log)
    ev = evaluate(net, test_mols, chunks_by_size(test_mols))
    rep = {"n_train": args.n_train, "n_train_converged": nconv, "n_pairs": int(pairs["X"].shape[0]), "epochs": args.epochs,
           "loss_history": hist, "n_test": ev["n"],
           "mean_iterations_sad": float(np.mean(ev["sad_iterations"])),
           "mean_iterations_learned": float(np.mean(ev["learned_iterations"])),
           "time_sad_s": ev["sad_s"], "time_learned_s": ev["learned_s"],
           "max_abs_dE": float(np.max(np.abs(ev["dE"]))), "fallbacks": ev["fallbacks"],
           "rms_density_error_sad": float(np.mean(ev["sad_err"])),
           "rms_density_error_learned": float(np.mean(ev["learned_err"])),
           "mean_abs_electron_count_error_learned": float(np.mean(np.abs(ev["learned_dN"]))),
           "wall_s": time.time() - t_start}
    log(json.dumps(rep))
    net.save(args.out)
    with open(os.path.splitext(args.out)[0] + ".json", "w") as fh:
        json.dump(rep, fh, indent=1)


if __name__ == "__main__":
    main()
