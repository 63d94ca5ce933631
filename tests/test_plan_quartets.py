"""Quartet planning (no GPU): plan_quartets against a brute-force enumeration of the
screened canonical quartets -- every quartet once, the Schwarz test, the diagonal
quartet always kept, the FP32 part of the mixed-precision split -- and the bucket
order of each class list."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from pychem_gb300.engine import plan_quartets


def _expand(plan, ket):
    out = {}
    rows = []
    for cls, part, bra, off, qs, dg in plan:
        for r in range(bra.numel()):
            n = int(off[r + 1] - off[r])
            rows.append((cls, part, int(bra[r]), int(qs[r])))
            for q in range(n):
                kp = int(bra[r]) if (dg[r] and q == n - 1) else int(ket[int(qs[r]) + q])
                assert (int(bra[r]), kp) not in out
                out[(int(bra[r]), kp)] = (cls, part)
    return out, rows


@pytest.mark.parametrize("trial", range(24))
def test_plan_matches_brute_force(trial):
    rng = np.random.default_rng(trial)
    npair, nmol, nk = int(rng.integers(1, 250)), int(rng.integers(1, 5)), int(rng.integers(1, 5))
    Q = torch.as_tensor(10 ** rng.uniform(-9, 1, npair))
    if trial % 3 == 0:
        Q[torch.as_tensor(rng.integers(0, npair, 5))] = float(Q[0])     # ties
    kind = torch.as_tensor(rng.integers(0, nk, npair))
    mol = torch.as_tensor(rng.integers(0, nmol, npair))
    ct = torch.as_tensor(rng.integers(0, 3, (nk, nk)))
    thr, thr32 = 1e-8, (1e-4 if trial % 2 else 0.0)
    work = torch.as_tensor(rng.integers(1, 5, nk)) if trial % 4 == 1 else None
    plan, ket = plan_quartets(Q, kind, mol, nmol, ct, thr, thr32, kind_work=work)
    got, rows = _expand(plan, ket)
    order = ket.numpy()
    posn = np.empty(npair, dtype=np.int64)
    posn[order] = np.arange(npair)
    Qn, kn, mn = Q.numpy(), kind.numpy(), mol.numpy()
    want = {}
    for p in range(npair):
        for q in range(npair):
            if mn[p] != mn[q] or kn[p] < kn[q] or (kn[p] == kn[q] and posn[q] > posn[p]):
                continue
            screened = Qn[p] * Qn[q] > thr
            if not (screened or p == q):
                continue
            fp32 = screened and thr32 > 0 and not Qn[p] * Qn[q] > thr32
            want[(p, q)] = (int(ct[kn[p], kn[q]]), "32" if fp32 else "64")
    assert got == want
    # within a class list the rows run in (-work, bra kind, ket kind, bra position) order
    wk = work.numpy() if work is not None else np.ones(nk, dtype=np.int64)
    for cls, part, bra, off, qs, dg in plan:
        keyr = [(-wk[kn[int(b)]] * wk[kn[order[int(s)]]], kn[int(b)], kn[order[int(s)]], posn[int(b)])
                for b, s in zip(bra, qs)]
        assert keyr == sorted(keyr)
