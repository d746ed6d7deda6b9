"""TEST INFRASTRUCTURE ONLY: a pure-Python restatement of the tree-level prover, for small cases.

It follows the reference's CPU prover level by level (crates/tessera-sumcheck/src/trees.rs:260-345
FractionTree, prove_trees :761; level.rs:127-262 the level sumcheck; crates/tessera-logup/src/
prover.rs:361 the leaf stage): at stage level l, forests joining at l draw root challenges
tree/l/root/c and take the last s of them as their point; γ (tree/l/gamma) and, with a fraction
tree present, λ (tree/l/lambda) are drawn; the present trees' claims are batched as
Σ γ^i·2^(n_max − n_i)·claim_i over one sumcheck of n_max rounds in which a tree of n_i < n_max
variables is front-padded; each round's message p_j(0), p_j(2), p_j(3) is absorbed under
tree/l/round/j and r_j drawn under tree/l/r/j; the final evaluations of every tree's tables go in
under tree/l/evals, and ρ (tree/l/line) moves each claim to the level below. Unlike the CUDA path
(which never tabulates eq and sums only q(0) and q(∞)), each round here is the textbook sum over the
bound tables and a bound eq table at X = 0, 2, 3 — a different route to the same field values.
Pure-Python loops: heights of a few levels only. The product package never imports this module.
"""
from __future__ import annotations

import struct

P = (1 << 64) - (1 << 32) + 1
W = 7


def add(a, b):
    return ((a[0] + b[0]) % P, (a[1] + b[1]) % P)


def sub(a, b):
    return ((a[0] - b[0]) % P, (a[1] - b[1]) % P)


def mul(a, b):
    return ((a[0] * b[0] + W * a[1] * b[1]) % P, (a[0] * b[1] + a[1] * b[0]) % P)


def scale(a, k: int):
    return (a[0] * k % P, a[1] * k % P)


ONE, ZERO = (1, 0), (0, 0)


def tce_fp2s(values) -> bytes:
    """TCE Vec<Fp2>: the count as u64 LE, then each (c0, c1) as two u64 LE."""
    return struct.pack("<Q", len(values)) + b"".join(struct.pack("<QQ", v[0], v[1]) for v in values)


def line(a, b, r):
    return add(a, mul(r, sub(b, a)))


def mle(values, point):
    """Σ_x values[x]·eq(point, x), x_1 the lowest bit, by binding one coordinate at a time (a
    joining forest's claim on its roots, crates/tessera-sumcheck/src/trees.rs:761 prove_trees)."""
    v = list(values)
    for r in point:
        v = [line(v[2 * i], v[2 * i + 1], r) for i in range(len(v) // 2)]
    return v[0]


def eq_table(point):
    """eq(point, x) = Π_k (x_k ? point[k] : 1 − point[k]) for every x (x_k bit k of the index)."""
    out = []
    for x in range(1 << len(point)):
        e = ONE
        for k, r in enumerate(point):
            e = mul(e, r if (x >> k) & 1 else sub(ONE, r))
        out.append(e)
    return out


def lagrange4(v, r):
    """The cubic through (0, v0), (1, v1), (2, v2), (3, v3) at r."""
    i2, i6 = pow(2, P - 2, P), pow(6, P - 2, P)
    r1, r2, r3 = sub(r, (1, 0)), sub(r, (2, 0)), sub(r, (3, 0))
    l0 = scale(mul(mul(r1, r2), r3), (P - i6) % P)
    l1 = scale(mul(mul(r, r2), r3), i2)
    l2 = scale(mul(mul(r, r1), r3), (P - i2) % P)
    l3 = scale(mul(mul(r, r1), r2), i6)
    return add(add(mul(l0, v[0]), mul(l1, v[1])), add(mul(l2, v[2]), mul(l3, v[3])))


class OTree:
    """One tree of a stage: a forest of 2^s product trees (kind 0) from 2^(s+h) Fp2 leaves, or a
    fraction tree (kind 1) from numerators (None: all 1) and denominators, with `sent` the root
    the roots message carried (None: its own). Levels are built as the reference's FractionTree
    and product trees build them (crates/tessera-sumcheck/src/trees.rs:260-300): entry x of a level
    from entries 2x and 2x + 1 below, (n, d) = (n_l·d_r + n_r·d_l, d_l·d_r) or the product."""

    def __init__(self, kind, s, leaves=None, numerators=None, denominators=None, sent=None):
        self.kind, self.s, self.sent = kind, s, sent
        if kind == 0:
            lv = [list(leaves)]
            while len(lv[0]) > (1 << s):
                below = lv[0]
                lv.insert(0, [mul(below[2 * x], below[2 * x + 1]) for x in range(len(below) // 2)])
            self.n = lv
            self.d = None
        else:
            nums = list(numerators) if numerators is not None else [ONE] * len(denominators)
            ln, ld = [nums], [list(denominators)]
            while len(ld[0]) > 1:
                n, d = ln[0], ld[0]
                ln.insert(0, [add(mul(n[2 * x], d[2 * x + 1]), mul(n[2 * x + 1], d[2 * x])) for x in range(len(d) // 2)])
                ld.insert(0, [mul(d[2 * x], d[2 * x + 1]) for x in range(len(d) // 2)])
            self.n, self.d = ln, ld
        self.h = len(self.n) - 1
        self.own = -1  # the tree's own level whose claim it holds (−1: not joined yet)
        self.point, self.value, self.p, self.q = [], ZERO, ZERO, ZERO

    def root(self):
        return self.n[0] if self.kind == 0 else (self.n[0][0], self.d[0][0])

    def tables(self, own):
        """The halves of the tree's level own + 1: (L, R) or (N0, N1, D0, D1)."""
        n = self.n[own + 1]
        if self.kind == 0:
            return [n[0::2], n[1::2]]
        d = self.d[own + 1]
        return [n[0::2], n[1::2], d[0::2], d[1::2]]

    def g(self, vals, lam):
        if self.kind == 0:
            return mul(vals[0], vals[1])
        n0, n1, d0, d1 = vals
        return add(add(mul(n0, d1), mul(n1, d0)), mul(lam, mul(d0, d1)))


class OStage:
    """A leaf stage over OTrees in schedule order (all leaves at stage level H)."""

    def __init__(self, trees):
        self.trees = trees
        self.H = max(t.h for t in trees)
        self.level = 0

    def prove_level(self, t) -> dict:
        """The stage's next level on transcript t (crates/tessera-sumcheck/src/trees.rs:761
        prove_trees, one ProvenTreeLevel; the batched level sumcheck of level.rs:127-262 with the
        padding of prover.rs:1122-1410), as a record of what it absorbed and drew."""
        level, H = self.level, self.H
        prefix = f"tree/{level}"
        joining = [k for k, tr in enumerate(self.trees) if H - tr.h == level]
        s_max = max([self.trees[k].s for k in joining if self.trees[k].kind == 0], default=0)
        rootc = [t.challenge_fp2(f"{prefix}/root/{c}") for c in range(s_max)]
        present = [k for k, tr in enumerate(self.trees) if tr.own >= 0 or H - tr.h == level]
        for k in joining:
            tr = self.trees[k]
            if tr.kind == 0:
                tr.point = rootc[s_max - tr.s:]
                tr.value = mle(tr.n[0], tr.point)
            else:
                tr.point = []
                tr.p, tr.q = tr.sent if tr.sent is not None else tr.root()
        gamma = t.challenge_fp2(f"{prefix}/gamma")
        fraction = any(self.trees[k].kind == 1 for k in present)
        lam = t.challenge_fp2(f"{prefix}/lambda") if fraction else None
        lm = lam or ZERO
        held, own_claim, tabs, eqs, nvars = [], [], [], [], []
        for k in present:
            tr = self.trees[k]
            own = max(tr.own, 0)
            if tr.kind == 0:
                held.append(tr.value)
                own_claim.append(tr.value)
            else:
                held.append(add(tr.p, mul(lm, tr.q)))
                rn, rd = tr.root()
                own_claim.append(add(rn, mul(lm, rd)) if tr.own < 0 else held[-1])
            tabs.append(tr.tables(own))
            eqs.append(eq_table(tr.point))
            nvars.append(len(tr.point))
        n_max = max(nvars, default=0)
        pads = [n_max - n for n in nvars]
        gpow = [ONE]
        for _ in present[1:]:
            gpow.append(mul(gpow[-1], gamma))
        claim = ZERO
        for i in range(len(present)):
            claim = add(claim, mul(gpow[i], scale(held[i], pow(2, pads[i], P))))
        claims, rounds, chal = [claim], [], []
        for j in range(n_max):
            msg = [ZERO, ZERO, ZERO]
            for i, k in enumerate(present):
                tr = self.trees[k]
                if j < pads[i]:
                    v = mul(gpow[i], scale(own_claim[i], pow(2, pads[i] - j - 1, P)))
                    msg = [add(m, v) for m in msg]
                    continue
                e, tb = eqs[i], tabs[i]
                for xi, X in enumerate((0, 2, 3)):
                    xs = (X, 0)
                    acc = ZERO
                    for pidx in range(len(e) // 2):
                        ex = line(e[2 * pidx], e[2 * pidx + 1], xs)
                        vals = [line(tab[2 * pidx], tab[2 * pidx + 1], xs) for tab in tb]
                        acc = add(acc, mul(ex, tr.g(vals, lm)))
                    msg[xi] = add(msg[xi], mul(gpow[i], acc))
            rounds.append(msg)
            t.absorb(f"{prefix}/round/{j}", tce_fp2s(msg))
            r = t.challenge_fp2(f"{prefix}/r/{j}")
            chal.append(r)
            claims.append(lagrange4([msg[0], sub(claims[-1], msg[0]), msg[1], msg[2]], r))
            for i in range(len(present)):
                if j >= pads[i]:
                    eqs[i] = [line(eqs[i][2 * p_], eqs[i][2 * p_ + 1], r) for p_ in range(len(eqs[i]) // 2)]
                    tabs[i] = [[line(tab[2 * p_], tab[2 * p_ + 1], r) for p_ in range(len(tab) // 2)] for tab in tabs[i]]
        evals = [tab[0] for tb in tabs for tab in tb]
        t.absorb(f"{prefix}/evals", tce_fp2s(evals))
        rho = t.challenge_fp2(f"{prefix}/line")
        cur = 0
        for i, k in enumerate(present):
            tr = self.trees[k]
            own_chal = chal[pads[i]:]
            if tr.kind == 0:
                u, w = evals[cur], evals[cur + 1]
                cur += 2
                tr.value = line(u, w, rho)
            else:
                n0, n1, d0, d1 = evals[cur:cur + 4]
                cur += 4
                tr.p, tr.q = line(n0, n1, rho), line(d0, d1, rho)
            tr.point = [rho] + list(own_chal)
            tr.own = max(tr.own, 0) + 1  # the claim now belongs to the tree's next level down
        self.level += 1
        return {"prefix": prefix, "root_challenges": rootc, "gamma": gamma, "lambda": lam, "rounds": rounds,
                "challenges": chal, "claims": claims, "final_evals": evals, "rho": rho, "present": present,
                "state": t.state.hex(), "counter": t.counter}

    def claim(self, k):
        tr = self.trees[k]
        return tr.point, (tr.value if tr.kind == 0 else (tr.p, tr.q))
