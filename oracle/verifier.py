"""TEST INFRASTRUCTURE ONLY: the independent verifier's checks, restated in Python.

The tests run every proof the CUDA path makes through these checks, so that acceptance by the
reference's verifier is checked, not assumed from byte equality with the oracle prover. Each
function follows the reference verifier (verifier/crates/...) step for step, in its own code:

- `next_claim`: a round polynomial known at 0, 1, ..., d evaluated at the challenge by Newton's
  forward differences (tv-core/src/interpolation.rs:58-80), p(1) = claim - p(0);
- `reduce`, `verify_batch`, `finish_batch`: the batched sumcheck (tv-core/src/sumcheck.rs:306-560):
  shape checks before the transcript moves, gamma, the padded claim sum, each round's message
  length, absorb and challenge, the final evaluations' count and absorb, and the relation sum
  against the last claim;
- `verify_level`: one level of the leaf stage (tv-core/src/tree.rs:132-420): gamma, lambda when a
  fraction tree is present, the batch with eq(r_i, r'_i)·g_i, then rho and the next claims;
- `check_roots`, `check_leaves`: LogUp's root and leaf checks (tv-core/src/logup.rs:359-560);
- `verify_leaf_stage`: the three LogUp steps around the levels, with the schedule (each tree
  joining at H - h, forests' root claims from tree/{l}/root/{c}) derived from public data;
- `verify_multiproof`: canonical Merkle multiproofs (tv-hash/src/merkle.rs:137-210);
- `verify_opening`: an advice opening's steps 6 and 8.1-8.3 (RFC-0011, as the reference's
  spec/vectors/pcs/README.md orders them; tv-core/src/opening.rs).

Rejections raise `Reject(reason, **detail)` with the reference's verdict names (Sumcheck,
Lookup, Evaluation, MerklePath, Proximity). The product package never imports this module.
"""
from __future__ import annotations

import struct

from . import trees as T
from .oracle import hash_domain

P = T.P
ZERO, ONE = T.ZERO, T.ONE
add, sub, mul = T.add, T.sub, T.mul
MAX_DEGREE = 7  # protocol/1 (tv-core/src/sumcheck.rs Protocol::One)


class Reject(Exception):
    """A verdict other than accept: `reason` and the detail the reference reports with it."""

    def __init__(self, reason: str, **detail):
        super().__init__(f"{reason} {detail}")
        self.reason, self.detail = reason, detail


# ---- field helpers --------------------------------------------------------------------------

def neg(a):
    return ((-a[0]) % P, (-a[1]) % P)


def inv(a):
    """1/a in Fp2 = Fp[X]/(X^2 - 7): conj(a)/norm(a)."""
    c0, c1 = a
    norm = (c0 * c0 - 7 * c1 * c1) % P
    ni = pow(norm, P - 2, P)
    return (c0 * ni % P, (-c1) * ni % P)


def fp(x: int):
    return (x % P, 0)


def eq(a, b):
    """eq(a, b) = Π_i (a_i b_i + (1 - a_i)(1 - b_i)), None for points of different lengths."""
    if len(a) != len(b):
        return None
    out = ONE
    for x, y in zip(a, b):
        xy = mul(x, y)
        out = mul(out, add(sub(sub(ONE, x), y), add(xy, xy)))
    return out


def tce(values) -> bytes:
    return T.tce_fp2s(values)


# ---- sumcheck -------------------------------------------------------------------------------

def next_claim(p0, rest, claim, r):
    """p(r) for the polynomial of degree d with p(0) = p0, p(1) = claim - p0, p(2..d) = rest:
    forward differences a_k = Δ^k p(0), then p(r) = a_0 + r/1·(a_1 + (r-1)/2·(a_2 + ...))."""
    values = [p0, sub(claim, p0)] + list(rest)
    diffs, row = [], values
    for _ in range(len(values)):
        diffs.append(row[0])
        row = [sub(row[i + 1], row[i]) for i in range(len(row) - 1)]
    acc = diffs[-1]
    for k in range(len(diffs) - 2, -1, -1):
        # acc ← a_k + (r − k)/(k + 1)·acc
        factor = mul(sub(r, fp(k)), fp(pow(k + 1, P - 2, P)))
        acc = add(diffs[k], mul(factor, acc))
    return acc


def reduce(t, prefix: str, degree: int, nvars: int, claim, rounds):
    """The rounds of one sumcheck: (point, last claim). Each round must be present and hold
    `degree` values; none may follow the last."""
    point = []
    for j in range(nvars):
        if j >= len(rounds):
            raise Reject("Sumcheck", check="missing round", round=j)
        msg = rounds[j]
        if len(msg) != degree:
            raise Reject("Sumcheck", check="round length", round=j)
        t.absorb(f"{prefix}/round/{j}", tce(msg))
        r = t.challenge_fp2(f"{prefix}/r/{j}")
        claim = next_claim(msg[0], msg[1:], claim, r)
        point.append(r)
    if len(rounds) > nvars:
        raise Reject("Sumcheck", check="extra round", round=nvars)
    return point, claim


def batch_shape(degree: int, sizes):
    """(degree, n_max, Σ k_i) of a batch whose instances have (n_i, k_i), checked before the
    transcript moves."""
    if not 1 <= degree <= MAX_DEGREE:
        raise Reject("Sumcheck", check="degree", degree=degree)
    sizes = list(sizes)
    if not sizes:
        raise Reject("Sumcheck", check="no instances")
    return degree, max(n for n, _ in sizes), sum(k for _, k in sizes)


def finish_batch(t, prefix: str, shape, gamma, instances, rounds, final_evals, relation):
    """Steps after γ: the padded claim Σ_i γ^i·2^(n_max − n_i)·c_i, the rounds, the evaluations'
    count and absorb, and Σ_i γ^i·relation_i against the last claim. instances: (claim, n_i,
    k_i) in schedule order; relation(i, own point, own evals) -> Fp2."""
    degree, n_max, expected = shape
    claim, w = ZERO, ONE
    for c, n, _ in instances:
        claim = add(claim, mul(w, T.scale(c, pow(2, n_max - n, P))))
        w = mul(w, gamma)
    point, last = reduce(t, prefix, degree, n_max, claim, rounds)
    if len(final_evals) != expected:
        raise Reject("Sumcheck", check="evaluation count", round=n_max)
    t.absorb(f"{prefix}/evals", tce(final_evals))
    value, w, at = ZERO, ONE, 0
    for i, (_, n, k) in enumerate(instances):
        own = point[len(point) - n:] if n else []
        got = relation(i, own, final_evals[at:at + k])
        if got is None:
            raise Reject("Sumcheck", check="relation", instance=i)
        at += k
        value = add(value, mul(w, got))
        w = mul(w, gamma)
    if value != last:
        raise Reject("Sumcheck", check="final", round=n_max)
    return point


def verify_batch(t, prefix: str, degree: int, instances, rounds, final_evals, relation):
    """A batched sumcheck under `prefix`: (γ, point). instances: (claim, n_i, k_i)."""
    shape = batch_shape(degree, [(n, k) for _, n, k in instances])
    gamma = t.challenge_fp2(f"{prefix}/gamma")
    point = finish_batch(t, prefix, shape, gamma, instances, rounds, final_evals, relation)
    return gamma, point


def product_relation(_i, _point, evals):
    out = ONE
    for e in evals:
        out = mul(out, e)
    return out


# ---- tree levels ----------------------------------------------------------------------------
# A claim is ("product", point, value) or ("fraction", point, numerator, denominator).

def _entering(c, lam):
    return c[2] if c[0] == "product" else add(c[2], mul(lam, c[3]))


def _k(c):
    return 2 if c[0] == "product" else 4


def verify_level(t, prefix: str, claims, rounds, final_evals):
    """One level of the leaf stage for the claims present, in schedule order: returns
    (γ, λ or None, point, ρ, next claims)."""
    shape = batch_shape(3, [(len(c[1]), _k(c)) for c in claims])
    gamma = t.challenge_fp2(f"{prefix}/gamma")
    lam = t.challenge_fp2(f"{prefix}/lambda") if any(c[0] == "fraction" for c in claims) else None
    lm = lam if lam is not None else ZERO
    instances = [(_entering(c, lm), len(c[1]), _k(c)) for c in claims]

    def relation(i, own, ev):
        c = claims[i]
        e = eq(c[1], own)
        if e is None or len(ev) != _k(c):
            return None
        if c[0] == "product":
            g = mul(ev[0], ev[1])
        else:
            n0, n1, d0, d1 = ev
            g = add(add(mul(n0, d1), mul(n1, d0)), mul(lm, mul(d0, d1)))
        return mul(e, g)

    point = finish_batch(t, prefix, shape, gamma, instances, rounds, final_evals, relation)
    rho = t.challenge_fp2(f"{prefix}/line")
    nxt, at = [], 0
    for c in claims:
        n = len(c[1])
        own = point[len(point) - n:] if n else []
        ev = final_evals[at:at + _k(c)]
        at += _k(c)
        if c[0] == "product":
            nxt.append(("product", [rho] + own, T.line(ev[0], ev[1], rho)))
        else:
            nxt.append(("fraction", [rho] + own, T.line(ev[0], ev[1], rho), T.line(ev[2], ev[3], rho)))
    return gamma, lam, point, rho, nxt


# ---- LogUp ----------------------------------------------------------------------------------

def check_roots(t, instances: int, roots):
    """α, β, the roots message (n_a, d_a, n_t, d_t per instance, absorbed whole) and each
    instance's d_a ≠ 0, d_t ≠ 0, n_a·d_t + n_t·d_a = 0. Returns (α, β, root claims)."""
    alpha = t.challenge_fp2("logup/alpha")
    beta = t.challenge_fp2("logup/beta")
    if len(roots) != 4 * instances:
        raise Reject("Lookup", check="roots length", instance=max(0, min(len(roots) // 4, instances - 1)))
    t.absorb("logup/roots", tce(roots))
    out = []
    for i in range(instances):
        n_a, d_a, n_t, d_t = roots[4 * i:4 * i + 4]
        if d_a == ZERO or d_t == ZERO or add(mul(n_a, d_t), mul(n_t, d_a)) != ZERO:
            raise Reject("Lookup", check="roots", instance=i)
        out.append((("fraction", [], n_a, d_a), ("fraction", [], n_t, d_t)))
    return alpha, beta, out


def check_leaves(t, alpha, beta, leaves, values, table):
    """The values message (one per instance whose table has values, absorbed whole), then per
    instance: the lookup tree's leaf numerator is 1 and the table tree's leaf denominator is
    α − t̃(ρ_t). leaves: (lookup claim, table claim, has_values). Returns, per instance, the key,
    value and multiplicity claims left for later stages."""
    expected = sum(1 for lf in leaves if lf[2])
    if len(values) != expected:
        raise Reject("Lookup", check="values length")
    t.absorb("logup/values", tce(values))
    sent = iter(values)
    out = []
    for i, (lookup, table_claim, has_values) in enumerate(leaves):
        v = next(sent) if has_values else None
        if lookup[2] != ONE:
            raise Reject("Lookup", check="leaf numerator", instance=i)
        if table_claim[3] != sub(alpha, table(i, table_claim[1])):
            raise Reject("Lookup", check="table evaluation", instance=i)
        key = sub(sub(alpha, lookup[3]), mul(beta, v if v is not None else ZERO))
        out.append({"key": (lookup[1], key), "value": (lookup[1], v) if v is not None else None,
                    "multiplicity": (table_claim[1], neg(table_claim[2]))})
    return out


def verify_leaf_stage(t, schedule, proofs, roots=None, values=None, tables=None):
    """The leaf stage on transcript t: LogUp's roots (when the stage has LogUp instances), every
    level, then LogUp's leaf checks. Every input is public, as the verifier holds it.

    schedule: entries in schedule order, each {"kind": "forest", "s": s, "h": h, "roots": [Fp2 ×
    2^s]} or {"kind": "lookup" | "table", "instance": i, "h": h}; proofs: one {"rounds",
    "final_evals"} per level; tables[i] = (rows as (key, value) pairs, has_values, h_t) for the
    table evaluation t̃ = kẽy + β·valũe with padding rows copies of row 0. Returns each schedule
    entry's leaf claim and the LogUp claims."""
    logup = sorted({e["instance"] for e in schedule if e["kind"] != "forest"})
    alpha = beta = None
    root_claims = {}
    if logup or roots is not None:
        alpha, beta, rc = check_roots(t, len(logup), roots or [])
        for i, (la, ta) in enumerate(rc):
            root_claims[(i, "lookup")], root_claims[(i, "table")] = la, ta
    H = max([e["h"] for e in schedule], default=0)
    held = {}
    for k, e in enumerate(schedule):
        if e["h"] == 0 and e["kind"] != "forest":
            held[k] = root_claims[(e["instance"], e["kind"])]
    for level in range(H):
        prefix = f"tree/{level}"
        joining = [k for k, e in enumerate(schedule) if H - e["h"] == level]
        s_max = max([schedule[k]["s"] for k in joining if schedule[k]["kind"] == "forest"], default=0)
        rootc = [t.challenge_fp2(f"{prefix}/root/{c}") for c in range(s_max)]
        for k in joining:
            e = schedule[k]
            if e["kind"] == "forest":
                pt = rootc[s_max - e["s"]:] if e["s"] else []
                held[k] = ("product", pt, T.mle(e["roots"], pt))
            else:
                held[k] = root_claims[(e["instance"], e["kind"])]
        present = [k for k, e in enumerate(schedule) if e["h"] > 0 and H - e["h"] <= level]
        if level >= len(proofs):
            raise Reject("Sumcheck", check=f"level {level}", instance=0, detail="missing level")
        pr = proofs[level]
        try:
            _, _, _, _, nxt = verify_level(t, prefix, [held[k] for k in present], pr["rounds"], pr["final_evals"])
        except Reject as r:
            raise Reject("Sumcheck", check=f"level {level}", instance=0, cause=r.detail) from None
        for k, c in zip(present, nxt):
            held[k] = c
    claims = {}
    if logup or values is not None:
        leaves = []
        for i in logup:
            la = next(held[k] for k, e in enumerate(schedule) if e["kind"] == "lookup" and e["instance"] == i)
            ta = next(held[k] for k, e in enumerate(schedule) if e["kind"] == "table" and e["instance"] == i)
            leaves.append((la, ta, tables[i][1]))

        def table_eval(i, point):
            rows, has_values, h_t = tables[i]
            padded = list(rows) + [rows[0]] * ((1 << h_t) - len(rows))
            return T.mle([add(fp(key), mul(beta, fp(val if has_values else 0))) for key, val in padded], point)

        claims = check_leaves(t, alpha, beta, leaves, values or [], table_eval)
    return held, claims


# ---- Merkle multiproofs ---------------------------------------------------------------------

def merkle_node(left: bytes, right: bytes) -> bytes:
    return hash_domain("merkle-node", left + right)


def verify_multiproof(root: bytes, n: int, leaves, siblings):
    """leaves: (index, digest) with strictly increasing indices below n; siblings: the digests
    the verifier cannot compute, level by level from the leaves up, left to right. Raises
    Reject("MerklePath") on the first failing check."""
    if n < 1 or n & (n - 1):
        raise Reject("MerklePath", check="tree size")
    if not leaves:
        raise Reject("MerklePath", check="no leaves")
    prev = -1
    for idx, _ in leaves:
        if idx <= prev:
            raise Reject("MerklePath", check="unordered")
        if idx >= n:
            raise Reject("MerklePath", check="out of range")
        prev = idx
    levels = n.bit_length() - 1
    # the canonical length, from the indices alone
    need, nodes = 0, sorted({i for i, _ in leaves})
    for _ in range(levels):
        s = set(nodes)
        need += sum(1 for x in nodes if x ^ 1 not in s)
        nodes = sorted({x >> 1 for x in nodes})
    if len(siblings) != need:
        raise Reject("MerklePath", check="sibling count")
    known = dict(leaves)
    at = 0
    for _ in range(levels):
        up = {}
        for x in sorted(known):
            if (x >> 1) in up:  # the right child of a pair already combined
                continue
            mate = x ^ 1
            if mate in known:
                other = known[mate]
            else:
                other = siblings[at]
                at += 1
            up[x >> 1] = merkle_node(known[x], other) if x & 1 == 0 else merkle_node(other, known[x])
        known = up
    if known.get(0) != root:
        raise Reject("MerklePath", check="root")


def canonical_multiproof(nodes, n: int, indices):
    """The canonical multiproof of `indices` from a tree's nodes (leaves first, root last, as
    merkle_tree lays them out): the prover's side, for assembling openings in tests."""
    out, base, width = [], 0, n
    cur = sorted(set(indices))
    while width > 1:
        s = set(cur)
        for x in cur:
            if x ^ 1 not in s:
                out.append(bytes(nodes[base + (x ^ 1)]))
        base += width
        width //= 2
        cur = sorted({x >> 1 for x in cur})
    return out


# ---- advice openings --------------------------------------------------------------------------

def _fp(x):
    return int(x, 16) if isinstance(x, str) else int(x)


def _f2(p):
    return (_fp(p[0]), _fp(p[1]))


def row_coefficients(op):
    """c_g(row) = Σ_{claims in g} γ·eq(row_point, row) for each group, then ξ_row = eq(ξ*, row),
    each over the non-zero rows in layout order."""
    rows = [r for seg in op["segments"] for r in seg]
    rv = op["row_vars"]

    def bits(r):
        return [fp((r >> t) & 1) for t in range(rv)]

    out = []
    for g in op["groups"]:
        cs = []
        for r in rows:
            c = ZERO
            for cl in g["claims"]:
                c = add(c, mul(_f2(cl["gamma"]), eq([_f2(x) for x in cl["row_point"]], bits(r))))
            cs.append(c)
        out.append(cs)
    xi = [_f2(x) for x in op["xi_point"]]
    out.append([eq(xi, bits(r)) for r in rows])
    return out


def _enc_at(u, x: int, k: int, n: int):
    """enc(u)(x) for x off H: Σ_i u_i·L_i(x), L_i(x) = (x^k − 1)·ω^i/(k·(x − ω^i)) (barycentric)."""
    w = pow(7, (P - 1) // k, P)
    zh = (pow(x, k, P) - 1) % P
    kinv = pow(k, P - 2, P)
    acc = ZERO
    wi = 1
    for i in range(k):
        li = zh * wi % P * kinv % P * pow((x - wi) % P, P - 2, P) % P
        acc = add(acc, T.scale(u[i], li))
        wi = wi * w % P
    return acc


def _mask_at(m, x: int):
    acc, xp = ZERO, 1
    for c in m:
        acc = add(acc, T.scale(c, xp))
        xp = xp * x % P
    return acc


def column_digest(commitment_id: bytes, j: int, symbols, block: int) -> bytes:
    """Column j's chain over its symbols (one per row, in row order): d_j[0] = H("column-init",
    id ‖ u64 j), then H("column-step", d ‖ the next `block` symbols) per block. An unmasked
    commitment's leaf j is this digest (crates/tessera-pcs/src/commitment.rs:343-458)."""
    d = hash_domain("column-init", commitment_id + struct.pack("<Q", j))
    for b in range(0, len(symbols), block):
        d = hash_domain("column-step", d + b"".join(struct.pack("<Q", int(s)) for s in symbols[b:b + block]))
    return d


def opening_leaf(op, j: int, column) -> bytes:
    """leaf_j from the column's symbols (one per non-zero row, layout order): each segment's chain
    d_j[0] = H("column-init", id ‖ u64 j), then a column-step per block of B rows; then
    H("column-merge", d^(1) ‖ ... ‖ d^(S))."""
    cid = bytes.fromhex(op["commitment_id"])
    B = op["row_block"]
    at, digests = 0, []
    for seg in op["segments"]:
        digests.append(column_digest(cid, j, column[at:at + len(seg)], B))
        at += len(seg)
    return hash_domain("column-merge", b"".join(digests))


def verify_opening(op):
    """An advice opening: step 6 (shape of the combined rows, then each group's sums), 8.1 (one
    column per distinct query, one symbol per non-zero row), 8.2 (leaves from the columns and the
    multiproof), 8.3 (each combined row against the columns at every distinct query)."""
    k = 1 << op["log2_k"]
    n = k << op["log2_inv_rate"]
    PA = op["mask_coeffs"]
    G = len(op["groups"])
    rows = [r for seg in op["segments"] for r in seg]
    comb = op["combined"]
    # 6: shape, then sums
    if len(comb) != G + 1 or any(len(c["u"]) != k or len(c["mask"]) != PA for c in comb):
        raise Reject("Evaluation", group=None, column=None)
    lk = op["log2_k"]
    for gi, g in enumerate(op["groups"]):
        claimed = ZERO
        for cl in g["claims"]:
            claimed = add(claimed, mul(_f2(cl["gamma"]), _f2(cl["value"])))
        cp = [_f2(x) for x in g["column_point"]]
        opened = ZERO
        for i in range(k):
            opened = add(opened, mul(_f2(comb[gi]["u"][i]), eq(cp, [fp((i >> t) & 1) for t in range(lk)])))
        if claimed != opened:
            raise Reject("Evaluation", group=gi, column=None)
    distinct = sorted(set(op["queries"]))
    smallest = min(op["queries"])
    # 8.1
    cols = op["columns"]
    if len(cols) != len(distinct) or any(len(c) != len(rows) for c in cols):
        raise Reject("MerklePath", group=None, column=smallest)
    colv = [[_fp(x) for x in c] for c in cols]
    # 8.2
    leaves = [(j, opening_leaf(op, j, colv[q])) for q, j in enumerate(distinct)]
    try:
        verify_multiproof(bytes.fromhex(op["root"]), n, leaves, [bytes.fromhex(s) for s in op["siblings"]])
    except Reject:
        raise Reject("MerklePath", group=None, column=smallest) from None
    # 8.3
    coeffs = row_coefficients(op)
    wn = pow(7, (P - 1) // n, P)
    for q, j in enumerate(distinct):
        x = 7 * pow(wn, j, P) % P
        zh = (pow(x, k, P) - 1) % P
        for gi in range(G + 1):
            lhs = ZERO
            for ri in range(len(rows)):
                lhs = add(lhs, T.scale(coeffs[gi][ri], colv[q][ri]))
            u = [_f2(v) for v in comb[gi]["u"]]
            m = [_f2(v) for v in comb[gi]["mask"]]
            rhs = add(_enc_at(u, x, k, n), T.scale(_mask_at(m, x), zh))
            if lhs != rhs:
                raise Reject("Proximity", group=None, column=j)
