"""Generate straight-line CUDA for the electron-repulsion classes (la lb|lc ld), l <= 2.

Scheme (Head-Gordon-Pople, as in the upstream integrals.py:427-555):
  primitive level:  Obara-Saika VRR building [e0|f0]^(0) for la <= |e| <= la+lb,
                    lc <= |f| <= lc+ld, bra first then ket; the contraction weights
                    are folded into the [00|00]^(m) prefactor so the contracted
                    accumulators are plain sums over primitive quartets;
  contracted level: bra HRR (a,b+1_i| = (a+1_i,b| + AB_i (a,b|, then ket HRR
                    |c,d+1_i) = |c+1_i,d) + CD_i |c,d);
  epilogue:         per-component normalisation ratio and Cartesian->spherical
                    rows (upstream Data/transform_basis.py:3-12) applied one index
                    at a time; identity for s and p shells.

The recurrence direction for a Cartesian triple is its first non-zero component
(x, then y, then z), the same choice as two_electron_vrr.c:33-48.  Only the nodes
reachable from the final targets are emitted (dead-code free), as SSA `const
double` statements the compiler keeps in registers.

Output: eri_gen.cuh (included by eri.cu).  Also reports FP64 operation counts per
class, which bench.py uses as the algorithmic work per primitive/contracted quartet.

    python pychem_gb300/csrc/gen_eri.py [--check]
"""
import json
import math
import os
import sys

LMAX = 2
HERE = os.path.dirname(os.path.abspath(__file__))


def carts(l):
    out = []
    for lx in range(l, -1, -1):
        for ly in range(l - lx, -1, -1):
            out.append((lx, ly, l - lx - ly))
    return out


def first_nz(t):
    for i in range(3):
        if t[i]:
            return i
    return -1


def dec(t, i, k=1):
    u = list(t)
    u[i] -= k
    return tuple(u)


def inc(t, i):
    u = list(t)
    u[i] += 1
    return tuple(u)


def pair_classes():
    return [(la, lb) for la in range(LMAX + 1) for lb in range(la + 1)]


def quartet_classes():
    pcs = pair_classes()
    out = []
    for i, bra in enumerate(pcs):
        for ket in pcs[: i + 1]:
            out.append(bra + ket)
    return out


def sph_rows(l):
    """Cartesian->spherical rows times the component normalisation ratio r_c
    (component scale relative to the pure-axis component, folded into cc)."""
    cs = carts(l)
    def scale(c):
        return (math.gamma(c[0] + 0.5) * math.gamma(c[1] + 0.5) * math.gamma(c[2] + 0.5)) ** -0.5
    pure = scale((l, 0, 0))
    ratio = [scale(c) / pure for c in cs]
    if l == 0:
        M = [[1.0]]
    elif l == 1:
        M = [[1.0, 0, 0], [0, 1.0, 0], [0, 0, 1.0]]
    elif l == 2:
        h = math.sqrt(3.0) / 2.0
        M = [[h, 0, 0, -h, 0, 0], [0, 1.0, 0, 0, 0, 0], [0, 0, 1.0, 0, 0, 0],
             [0, 0, 0, 0, 1.0, 0], [-0.5, 0, 0, -0.5, 0, 1.0]]
    else:
        raise ValueError(l)
    return [[M[r][c] * ratio[c] for c in range(len(cs))] for r in range(len(M))]


class Emitter:
    def __init__(self):
        self.lines = []
        self.nflop = 0      # FP64 operations (FMA counted as 1 instruction here)
        self.names = {}
        self.counter = 0

    def new(self, prefix="t"):
        self.counter += 1
        return "%s%d" % (prefix, self.counter)


def gen_vrr(la, lb, lc, ld, em, ctype="double"):
    """Emit VRR statements; returns dict target(e,f) -> variable name (m=0)."""
    L = la + lb + lc + ld
    memo = {}
    consts = set()

    def node(e, f, m):
        key = (e, f, m)
        if key in memo:
            return memo[key]
        if sum(e) == 0 and sum(f) == 0:
            name = "F%d" % m
            memo[key] = name
            return name
        terms = []
        if sum(f) == 0:
            i = first_nz(e)
            e1 = dec(e, i)
            a = node(e1, f, m)
            b = node(e1, f, m + 1)
            terms.append(("PA%s" % "xyz"[i], a))
            terms.append(("WP%s" % "xyz"[i], b))
            if e1[i] > 0:
                e2 = dec(e1, i)
                c = node(e2, f, m)
                d = node(e2, f, m + 1)
                consts.add(("oo2z", e1[i]))
                inner = em.new()
                em.lines.append("const %s %s = fma(-rz, %s, %s);" % (ctype, inner, d, c))
                em.nflop += 1
                terms.append(("oo2z_%d" % e1[i], inner))
        else:
            i = first_nz(f)
            f1 = dec(f, i)
            a = node(e, f1, m)
            b = node(e, f1, m + 1)
            terms.append(("QC%s" % "xyz"[i], a))
            terms.append(("WQ%s" % "xyz"[i], b))
            if f1[i] > 0:
                f2 = dec(f1, i)
                c = node(e, f2, m)
                d = node(e, f2, m + 1)
                consts.add(("oo2e", f1[i]))
                inner = em.new()
                em.lines.append("const %s %s = fma(-re, %s, %s);" % (ctype, inner, d, c))
                em.nflop += 1
                terms.append(("oo2e_%d" % f1[i], inner))
            if e[i] > 0:
                e1 = dec(e, i)
                g = node(e1, f1, m + 1)
                consts.add(("oo2ze", e[i]))
                terms.append(("oo2ze_%d" % e[i], g))
        name = em.new("v")
        expr = "%s * %s" % terms[0]
        for coef, var in terms[1:]:
            expr = "fma(%s, %s, %s)" % (coef, var, expr)
        em.lines.append("const %s %s = %s;" % (ctype, name, expr))
        em.nflop += len(terms)
        memo[key] = name
        return name

    targets = {}
    for le in range(la, la + lb + 1):
        for lf in range(lc, lc + ld + 1):
            for e in carts(le):
                for f in carts(lf):
                    targets[(e, f)] = node(e, f, 0)
    return targets, consts, L


def gen_hrr(la, lb, lc, ld, acc_name, em, ctype="double"):
    """Emit HRR from accumulators acc_name[(e,f)] to Cartesian (ab|cd) names."""
    memo = {}

    def node(a, b, c, d):
        key = (a, b, c, d)
        if key in memo:
            return memo[key]
        if sum(b) == 0 and sum(d) == 0:
            name = acc_name[(a, c)]
        elif sum(b) != 0:
            i = first_nz(b)
            b1 = dec(b, i)
            x = node(inc(a, i), b1, c, d)
            y = node(a, b1, c, d)
            name = em.new("h")
            em.lines.append("const %s %s = fma(AB%s, %s, %s);" % (ctype, name, "xyz"[i], y, x))
            em.nflop += 1
        else:
            i = first_nz(d)
            d1 = dec(d, i)
            x = node(a, b, inc(c, i), d1)
            y = node(a, b, c, d1)
            name = em.new("h")
            em.lines.append("const %s %s = fma(CD%s, %s, %s);" % (ctype, name, "xyz"[i], y, x))
            em.nflop += 1
        memo[key] = name
        return name

    out = {}
    for a in carts(la):
        for b in carts(lb):
            for c in carts(lc):
                for d in carts(ld):
                    out[(a, b, c, d)] = node(a, b, c, d)
    return out


def gen_sph(la, lb, lc, ld, cart, em, ctype="double"):
    """Apply the spherical rows index by index; returns list of output names in
    row-major (i,j,k,l) spherical order."""
    ls = [la, lb, lc, ld]
    cur = {}
    cidx = [carts(l) for l in ls]
    for a_i, a in enumerate(cidx[0]):
        for b_i, b in enumerate(cidx[1]):
            for c_i, c in enumerate(cidx[2]):
                for d_i, d in enumerate(cidx[3]):
                    cur[(a_i, b_i, c_i, d_i)] = cart[(a, b, c, d)]
    dims = [len(c) for c in cidx]
    for s in range(4):
        if ls[s] <= 1:
            continue
        rows = sph_rows(ls[s])
        nxt = {}
        for key in list(cur.keys()):
            if key[s] != 0:
                continue
            for r, row in enumerate(rows):
                terms = [(coef, cur[key[:s] + (c,) + key[s + 1:]]) for c, coef in enumerate(row) if coef != 0.0]
                name = em.new("s")
                if len(terms) == 1 and terms[0][0] == 1.0:
                    nxt[key[:s] + (r,) + key[s + 1:]] = terms[0][1]
                    continue
                lit = (lambda c: "%.9ef" % c) if ctype == "float" else (lambda c: "%.17g" % c)
                expr = "%s * %s" % (lit(terms[0][0]), terms[0][1])
                em.nflop += 1
                for coef, var in terms[1:]:
                    expr = "fma(%s, %s, %s)" % (lit(coef), var, expr)
                    em.nflop += 1
                em.lines.append("const %s %s = %s;" % (ctype, name, expr))
                nxt[key[:s] + (r,) + key[s + 1:]] = name
        cur = nxt
        dims[s] = len(rows)
    ns = [2 * l + 1 for l in ls]
    out = []
    for i in range(ns[0]):
        for j in range(ns[1]):
            for k in range(ns[2]):
                for l in range(ns[3]):
                    out.append(cur[(i, j, k, l)])
    return out


def count_flops(lines):
    """Floating-point operations of emitted statements: FMA = 2, MUL/ADD = 1."""
    total = 0
    for line in lines:
        total += 2 * line.count("fma(")
        total += line.count(" * ")
        total += line.count(" += ")
    return total


def overhead_flops(L):
    """Per primitive quartet, outside the VRR (see k_eri in eri_kernels.cuh): P-Q (3),
    zeta+eta (1), Newton rsqrt (9), 1/(zeta+eta) (1), rho (2), T (6), Boys top order
    (2 + 7 FMA), prefactor (2), scaling F_0..F_L (L+1); for L > 0 also exp(-T) (7 FMA
    + 2), downward recursion (3 per order) and the W-P, W-Q, 1/2(zeta+eta), rho/zeta,
    rho/eta factors (11)."""
    return 41 + L if L == 0 else 68 + 4 * L


def gen_class(la, lb, lc, ld, ctype="double", suffix=""):
    """Returns (source, stats) for the device functions of one class."""
    tag = "%d%d%d%d" % (la, lb, lc, ld)
    em = Emitter()
    targets, consts, L = gen_vrr(la, lb, lc, ld, em, ctype)
    vrr_lines, vrr_flop = em.lines, em.nflop
    acc_keys = sorted(targets.keys())
    acc_name = {k: "acc%d" % i for i, k in enumerate(acc_keys)}

    uses = {}
    for line in vrr_lines:
        for tok in ("PAx", "PAy", "PAz", "WPx", "WPy", "WPz", "QCx", "QCy", "QCz", "WQx", "WQy", "WQz", "rz", "re"):
            if tok in line:
                uses[tok] = True
    src = []
    fn = "eri_prim_%s%s" % (tag, suffix)
    nacc = len(acc_keys)
    src.append("// (%d%d|%d%d): L=%d, %d accumulators, %d VRR ops per primitive quartet"
               % (la, lb, lc, ld, L, nacc, vrr_flop + nacc))
    src.append("struct Eri%s%s {" % (tag, suffix))
    src.append("  static constexpr int L = %d;" % L)
    src.append("  static constexpr int NACC = %d;" % nacc)
    src.append("  static constexpr int NOUT = %d;" % ((2 * la + 1) * (2 * lb + 1) * (2 * lc + 1) * (2 * ld + 1)))
    src.append("  static constexpr int LA = %d, LB = %d, LC = %d, LD = %d;" % (la, lb, lc, ld))
    # primitive accumulate
    src.append("  template <class PQ> __device__ __forceinline__ static void prim(const PQ& q, const %s* F, %s* acc) {" % (ctype, ctype))
    for m in range(L + 1):
        src.append("    const %s F%d = F[%d];" % (ctype, m, m))
    for tok in sorted(uses):
        src.append("    const %s %s = q.%s;" % (ctype, tok, tok))
    for kind, k in sorted(consts):
        base = {"oo2z": "q.oo2z", "oo2e": "q.oo2e", "oo2ze": "q.oo2ze"}[kind]
        if k == 1:
            src.append("    const %s %s_1 = %s;" % (ctype, kind, base))
        else:
            src.append("    const %s %s_%d = %s(%d) * %s;" % (ctype, kind, k, ctype, k, base))
    for line in vrr_lines:
        src.append("    " + line)
    for k in acc_keys:
        src.append("    acc[%d] += %s;" % (acc_keys.index(k), targets[k]))
    src.append("  }")
    # contracted epilogue: HRR + spherical
    em2 = Emitter()
    cart = gen_hrr(la, lb, lc, ld, {k: "acc[%d]" % i for i, k in enumerate(acc_keys)}, em2, ctype)
    outs = gen_sph(la, lb, lc, ld, cart, em2, ctype)
    src.append("  template <class OutFn> __device__ __forceinline__ static void finish(const %s* acc, %s ABx, %s ABy, %s ABz, %s CDx, %s CDy, %s CDz, OutFn&& out) {"
               % ((ctype,) * 7))
    for line in em2.lines:
        src.append("    " + line)
    for i, name in enumerate(outs):
        src.append("    out(%d, %s);" % (i, name))
    src.append("  }")
    src.append("};")
    acc_lines = ["acc += v"] * nacc
    stats = dict(cls=tag, L=L, nacc=nacc, vrr_ops=vrr_flop + nacc, finish_ops=em2.nflop,
                 vrr_flops=count_flops(vrr_lines) + nacc, finish_flops=count_flops(em2.lines),
                 overhead_flops=overhead_flops(L),
                 nout=(2 * la + 1) * (2 * lb + 1) * (2 * lc + 1) * (2 * ld + 1))
    return "\n".join(src), stats


def main():
    parts = ["// Generated by gen_eri.py -- do not edit.",
             "// Straight-line HGP electron-repulsion classes (la lb|lc ld), l <= %d." % LMAX,
             "#pragma once", ""]
    stats = []
    for (la, lb, lc, ld) in quartet_classes():
        s, st = gen_class(la, lb, lc, ld, "double", "")
        parts.append(s)
        parts.append("")
        stats.append(st)
    for (la, lb, lc, ld) in quartet_classes():
        s, st = gen_class(la, lb, lc, ld, "float", "f")
        parts.append(s)
        parts.append("")
    text = "\n".join(parts) + "\n"
    out = os.path.join(HERE, "eri_gen.cuh")
    if "--check" in sys.argv:
        with open(out) as fh:
            if fh.read() != text:
                print("eri_gen.cuh is stale")
                sys.exit(1)
        return
    with open(out, "w") as fh:
        fh.write(text)
    with open(os.path.join(HERE, "eri_ops.json"), "w") as fh:
        json.dump(stats, fh, indent=0)
    for st in stats:
        print(st)


if __name__ == "__main__":
    main()
