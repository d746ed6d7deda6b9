"""Tree levels on the GPU against the reference's golden vectors: every product-tree batch,
product-forest batch and LogUp leaf stage of sumcheck.json, level by level — root challenges, γ, λ,
round messages, challenges, the verifier's claims, final evaluations, ρ, the claims each tree
carries to the next level, and the transcript state after every level."""
import gzip
import json
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

P = 0xFFFFFFFF00000001
W = 7
TREES = json.load(gzip.open(Path(__file__).parent / "golden" / "trees.json.gz"))


@pytest.fixture(scope="module")
def dev():
    from tessera_gb300.device import default_device

    return default_device()


def num(x):
    return int(x, 16)


def f2(pair):
    return (num(pair[0]), num(pair[1]))


def f2s(items):
    return [f2(p) for p in items]


def add(a, b):
    return ((a[0] + b[0]) % P, (a[1] + b[1]) % P)


def sub(a, b):
    return ((a[0] - b[0]) % P, (a[1] - b[1]) % P)


def mul(a, b):
    return ((a[0] * b[0] + W * a[1] * b[1]) % P, (a[0] * b[1] + a[1] * b[0]) % P)


def words(elems):
    return np.array([w for e in elems for w in e], dtype=np.uint64)


def transcript(ctx):
    from golden_data import context_tce
    from tessera_gb300.hash import Transcript

    return Transcript(context_tce(ctx))


def check_level(rec, want, stage, label):
    assert rec.prefix == want["prefix"], label
    assert rec.root_challenges == f2s(want.get("root_challenges", [])), label
    assert rec.gamma == f2(want["gamma"]), label
    if "lambda" in want:
        assert rec.lambda_ == (None if want["lambda"] is None else f2(want["lambda"])), label
    assert rec.rounds == [f2s(m) for m in want["rounds"]], label
    assert rec.challenges == f2s(want["challenges"]), label
    assert rec.claims == f2s(want["claims"]), label
    assert rec.final_evals == f2s(want["final_evals"]), label
    assert rec.rho == f2(want["rho"]), label
    assert rec.state.hex() == want["state"] and rec.counter == want["counter"], label
    key = "tree" if "tree" in want["next"][0] else "forest"
    assert [n[key] for n in want["next"]] == rec.present, label
    for n in want["next"]:
        point, claim, _ = stage.claim(n[key])
        assert point == f2s(n["point"]), label
        if "value" in n:
            assert claim == f2(n["value"]), label
        else:
            assert claim == (f2(n["numerator"]), f2(n["denominator"])), label


def leaf_table(values, base, on_device):
    """Prime-field leaves as Fp2 pairs, or as words (base); on the device when asked."""
    from tessera_gb300.trees import lift

    a = np.array(values, dtype=np.uint64) if base else lift(values)
    if not on_device:
        return a
    import torch

    return torch.from_numpy(a.view(np.int64)).cuda()


def forest_of(spec, base=False, on_device=False):
    from tessera_gb300.trees import Forest

    return Forest(spec["rows_log"], leaf_table([num(x) for x in spec["leaves"]], base, on_device), base)


# Fp2 leaves from the host; prime-field leaves (the forest's levels stay in the prime field) from
# the host and read in place on the device
LEAF_FORMS = [(False, False), (True, False), (True, True)]


@pytest.mark.parametrize("base,on_device", LEAF_FORMS)
def test_tree_batches(dev, base, on_device):
    from tessera_gb300.trees import Forest, LeafStage

    for b in TREES["tree_batches"]:
        t = transcript(b["context"])
        trees = [Forest(0, leaf_table([num(x) for x in tr["leaves"]], base, on_device), base) for tr in b["trees"]]
        with LeafStage(trees, dev) as st:
            for k, tr in enumerate(b["trees"]):
                assert st.root(k) == [(num(tr["root"]), 0)], b["name"]
            assert st.height == len(b["levels"])
            for want in b["levels"]:
                check_level(st.prove_level(t), want, st, b["name"])


@pytest.mark.parametrize("base,on_device", LEAF_FORMS)
def test_forest_batches(dev, base, on_device):
    from tessera_gb300.trees import LeafStage

    for b in TREES["forest_batches"]:
        t = transcript(b["context"])
        with LeafStage([forest_of(f, base, on_device) for f in b["forests"]], dev) as st:
            for k, f in enumerate(b["forests"]):
                assert st.root(k) == [(num(x), 0) for x in f["roots"]], b["name"]
            for want in b["levels"]:
                check_level(st.prove_level(t), want, st, b["name"])


def compress(beta, row):
    return add((row[0], 0), mul(beta, (row[1], 0)))


def mle(values, point):
    """Σ_x v[x]·eq(point, x), x_1 the lowest bit."""
    out = (0, 0)
    for x, v in enumerate(values):
        e = (1, 0)
        for i, r in enumerate(point):
            e = mul(e, r if (x >> i) & 1 else sub((1, 0), r))
        out = add(out, mul(v, e))
    return out


def logup_trees(alpha, beta, inst):
    """The honest prover's two fraction trees of an instance, from its description."""
    from tessera_gb300.trees import Fraction

    rows = [(num(k), num(v)) for k, v in inst["rows"]]
    tuples = [rows[j] if isinstance(j, int) else (num(j[0]), num(j[1])) for j in inst["lookups"]]
    h_a, h_t = inst["h_a"], inst["h_t"]
    slots = tuples + [rows[0]] * ((1 << h_a) - len(tuples))
    lookup_d = [sub(alpha, compress(beta, tp)) for tp in slots]
    m = [num(x) for x in inst["multiplicities"]]
    table_rows = rows + [rows[0]] * ((1 << h_t) - len(rows))
    table_n = [((P - mj) % P, 0) for mj in m]
    table_d = [sub(alpha, compress(beta, r)) for r in table_rows]
    values = [(tp[1], 0) for tp in slots]
    return Fraction(words(lookup_d)), Fraction(words(table_d), words(table_n)), values


HONEST_OR_DESCRIBED = ("accept", "roots", "level")


def test_logup_leaf_stages(dev):
    """Every LogUp batch whose prover data the vectors describe (the honest ones, and the cheats
    that change only lookups, multiplicities or the roots message): α and β, the roots message,
    each level of the leaf stage, the values message and the final transcript state."""
    from tessera_gb300.trees import LeafStage

    checked = 0
    for b in TREES["logup_batches"]:
        exp = b["expected"]
        kind = "accept" if exp == "accept" else ("roots" if exp.get("check") == "roots" else
                                                  "level" if str(exp.get("check", "")).startswith("level") else "other")
        if kind not in HONEST_OR_DESCRIBED:
            continue  # cheats on numerators, the table or its padding: the vectors do not describe that prover
        t = transcript(b["context"])
        alpha = t.challenge_fp2("logup/alpha")
        beta = t.challenge_fp2("logup/beta")
        assert (alpha, beta) == (f2(b["alpha"]), f2(b["beta"])), b["name"]
        built = [logup_trees(alpha, beta, inst) for inst in b["instances"]]
        sent = f2s(b["roots"])
        t.absorb_fp2s("logup/roots", sent)
        schedule = []
        for entry in b["trees"]:
            if entry["kind"] == "forest":
                schedule.append(forest_of(b["forests"][entry["index"]]))
            else:
                i, side = entry["index"], 0 if entry["kind"] == "lookup" else 1
                tree = built[i][side]
                tree.sent = (sent[4 * i + 2 * side], sent[4 * i + 2 * side + 1])
                schedule.append(tree)
        with LeafStage(schedule, dev) as st:
            for want in b["levels"]:
                check_level(st.prove_level(t), want, st, b["name"])
            place = {(e["kind"], e["index"]): k for k, e in enumerate(b["trees"])}
            values = []
            for i, inst in enumerate(b["instances"]):
                point_a, (p_a, q_a), _ = st.claim(place[("lookup", i)])
                point_t, (p_t, q_t), _ = st.claim(place[("table", i)])
                lc = b["leaf_checks"][i]
                assert point_a == f2s(lc["lookup"]["point"]) and (p_a, q_a) == (f2(lc["lookup"]["numerator"]),
                                                                              f2(lc["lookup"]["denominator"])), b["name"]
                assert point_t == f2s(lc["table"]["point"]) and (p_t, q_t) == (f2(lc["table"]["numerator"]),
                                                                             f2(lc["table"]["denominator"])), b["name"]
                if inst["has_values"]:
                    values.append(mle(built[i][2], point_a))
        assert values == f2s(b["values"]), b["name"]
        t.absorb_fp2s("logup/values", values)
        assert t.state.hex() == b["state"] and t.counter == b["counter"], b["name"]
        checked += 1
    assert checked >= 12


def counter_value(c):
    m = 2**64 - 1
    z = (c * 0x9E3779B97F4A7C15 + 0x9E3779B97F4A7C15) & m
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & m
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & m
    z ^= z >> 31
    return z - P if z >= P else z


@pytest.mark.parametrize("unit,h", [(True, 1), (False, 2), (True, 3), (False, 5), (True, 9), (False, 9), (True, 14),
                                    (False, 17)])
def test_generated_leaves_and_leaf_claims(dev, unit, h):
    """Generated LogUp leaves equal the counter generator's on the host; every level passes the
    verifier's last check (its last claim is eq(point, r)·(N0·D1 + N1·D0 + λ·D0·D1) at the final
    evaluations, which fails if any round message is wrong); and after the last level the final
    claims are the leaves' numerators' and denominators' MLEs at the final point (the verifier's
    leaf check). Heights past 12 run launched rounds as well as each level's single-block tail."""
    from tessera_gb300.hash import Mode, SessionContext, Transcript
    from tessera_gb300.trees import LeafStage, generated_fraction

    ks, vs, ms = 1000, 2000000, 77
    alpha, beta = (123456789, 987654321), (55555, 4444444)
    tree = generated_fraction(h, ks, vs, None if unit else ms, alpha, beta, dev)
    assert (tree.numerators is None) == unit
    n = np.tile(np.array([1, 0], dtype=np.uint64), 1 << h) if unit else tree.numerators.cpu().numpy().view(np.uint64)
    d = tree.denominators.cpu().numpy().view(np.uint64)
    for j in range(1 << h):
        k, v = counter_value(ks + j), counter_value(vs + j)
        assert (int(d[2 * j]), int(d[2 * j + 1])) == sub(alpha, add((k, 0), mul(beta, (v, 0))))
        m = counter_value(ms + j) & 0xFFFF
        assert (int(n[2 * j]), int(n[2 * j + 1])) == ((1, 0) if unit else ((P - m) % P, 0))
    t = Transcript(SessionContext("tessera-protocol/1", Mode.NON_INTERACTIVE, "test-small/1", bytes(32), bytes(16)))
    with LeafStage([tree], dev) as st:
        recs = st.prove(t)
        point, (p, q), own = st.claim(0)
    assert own == h and len(point) == h
    pt = []
    for rec in recs:
        n0, n1, d0, d1 = rec.final_evals
        g = add(add(mul(n0, d1), mul(n1, d0)), mul(rec.lambda_, mul(d0, d1)))
        assert rec.claims[-1] == mul(eq_at(pt, rec.challenges), g), rec.prefix
        pt = [rec.rho] + list(rec.challenges)
    nums = [(int(n[2 * j]), int(n[2 * j + 1])) for j in range(1 << h)]
    dens = [(int(d[2 * j]), int(d[2 * j + 1])) for j in range(1 << h)]
    assert (p, q) == (fold_mle(nums, point), fold_mle(dens, point))


def fold_mle(values, point):
    """The MLE of a table at a point by binding one coordinate at a time (x_1 the lowest bit)."""
    v = list(values)
    for r in point:
        v = [add(v[2 * i], mul(r, sub(v[2 * i + 1], v[2 * i]))) for i in range(len(v) // 2)]
    assert len(v) == 1
    return v[0]


def test_counter_fill(dev):
    """The device counter generator equals the host's, word for word (the reference's fill_counter)."""
    import torch

    from tessera_gb300.workloads import counter_words, fill_counter

    base = 1 << 61
    got = fill_counter(torch.empty(5000, dtype=torch.int64, device="cuda"), base, dev).cpu().numpy().view(np.uint64)
    assert np.array_equal(got, counter_words(base, 5000))
    assert [int(x) for x in got[:3]] == [counter_value(base + j) for j in range(3)]


def eq_at(p, r):
    out = (1, 0)
    for a, b in zip(p, r):
        out = mul(out, add(mul(a, b), mul(sub((1, 0), a), sub((1, 0), b))))
    return out


@pytest.mark.parametrize("s,h", [(4, 8), (0, 11), (7, 3), (6, 9), (2, 14), (12, 3), (6, 14), (3, 1)])
def test_prime_field_forest_matches_fp2_and_leaf_claim(dev, s, h):
    """A forest of counter leaves proven from prime-field words (read in place on the device) and
    from Fp2 pairs gives the same records level by level; every level passes the verifier's last
    check (the last round's claim is eq(point, r)·L(r)·R(r), which fails if any round message is
    wrong); the final claim is the leaves' MLE at the final point; and a second stage of the same
    shape, from the device's workspace cache, repeats the proof exactly."""
    import torch

    from tessera_gb300.hash import Mode, SessionContext, Transcript
    from tessera_gb300.trees import Forest, LeafStage, lift
    from tessera_gb300.workloads import fill_counter

    ctx = SessionContext("tessera-protocol/1", Mode.NON_INTERACTIVE, "test-small/1", bytes([7]) * 32, bytes([9]) * 16)
    leaves = fill_counter(torch.empty(1 << (s + h), dtype=torch.int64, device="cuda"), 1 << 61, dev)
    host = leaves.cpu().numpy().view(np.uint64)
    runs = []
    for forest in (Forest(s, leaves, True), Forest(s, lift(host)), Forest(s, leaves, True)):
        t = Transcript(ctx)
        with LeafStage([forest], dev) as st:
            recs = st.prove(t)
            runs.append(([(r.rounds, r.challenges, r.final_evals, r.rho) for r in recs], st.claim(0), t.state))
    assert runs[0] == runs[1] == runs[2]
    pt = None
    for k, (rounds, chal, evals, rho) in enumerate(runs[0][0]):
        pt = list(recs[k].root_challenges) if k == 0 else pt
        assert recs[k].claims[-1] == mul(eq_at(pt, chal), mul(evals[0], evals[1])), k
        pt = [rho] + list(chal)
    point, value, own = runs[0][1]
    assert own == h and len(point) == s + h
    assert value == fold_mle([(int(x), 0) for x in host], point)
    dev.trim()


def test_unaligned_device_leaves_are_copied(dev):
    """Prime-field leaves at an address that is not 16-byte aligned (a view one word into a
    tensor) cannot be read in place as word pairs: the stage copies them, and the proof equals the
    one from aligned leaves."""
    import torch

    from tessera_gb300.hash import Mode, SessionContext, Transcript
    from tessera_gb300.trees import Forest, LeafStage
    from tessera_gb300.workloads import fill_counter

    s, h = 3, 7
    ctx = SessionContext("tessera-protocol/1", Mode.NON_INTERACTIVE, "test-small/1", bytes([3]) * 32, bytes([4]) * 16)
    aligned = fill_counter(torch.empty(1 << (s + h), dtype=torch.int64, device="cuda"), 5, dev)
    backing = torch.zeros((1 << (s + h)) + 1, dtype=torch.int64, device="cuda")
    shifted = backing[1:]
    shifted.copy_(aligned)
    assert shifted.data_ptr() % 16 == 8
    out = []
    for leaves in (aligned, shifted):
        t = Transcript(ctx)
        with LeafStage([Forest(s, leaves, True)], dev) as st:
            recs = st.prove(t)
            out.append(([(r.rounds, r.final_evals) for r in recs], st.claim(0), t.state))
    assert out[0] == out[1]


def test_workspace_cache_reuse_and_trim(dev):
    """Stages of alternating shapes take their levels and bound tables from the device's workspace
    cache (buffers a closed stage left, possibly written by another shape) and prove exactly as the
    first time; tg_device_trim returns the cached memory to the driver."""
    import torch

    from tessera_gb300.hash import Mode, SessionContext, Transcript
    from tessera_gb300.trees import Forest, LeafStage, generated_fraction
    from tessera_gb300.workloads import fill_counter

    ctx = SessionContext("tessera-protocol/1", Mode.NON_INTERACTIVE, "test-small/1", bytes([5]) * 32, bytes([6]) * 16)
    big = fill_counter(torch.empty(1 << 22, dtype=torch.int64, device="cuda"), 11, dev)
    small = fill_counter(torch.empty(1 << 16, dtype=torch.int64, device="cuda"), 12, dev)

    def forest(leaves, s):
        t = Transcript(ctx)
        with LeafStage([Forest(s, leaves, True)], dev) as st:
            recs = st.prove(t)
            return [(r.rounds, r.final_evals) for r in recs], st.claim(0), t.state

    def fraction():
        t = Transcript(ctx)
        tree = generated_fraction(15, 3, 4, 5, (7, 8), (9, 10), dev)
        with LeafStage([tree], dev) as st:
            recs = st.prove(t)
            return [(r.rounds, r.final_evals) for r in recs], st.claim(0), t.state

    first = (forest(big, 8), forest(small, 4), fraction())
    for _ in range(2):
        assert (forest(big, 8), forest(small, 4), fraction()) == first
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    dev.trim()
    free_after = torch.cuda.mem_get_info()[0]
    assert free_after > free_before  # the 2^22-leaf forest's levels and tables went back


def test_leaf_stage_refusals(dev):
    """Malformed stages are refused before anything runs (unknown kind, too many variables, a
    fraction tree with s > 0 or prime-field leaves, missing leaves), and a level past the last one
    is refused with the transcript unchanged."""
    import ctypes

    from tessera_gb300 import _native as N
    from tessera_gb300.hash import Mode, SessionContext, Transcript
    from tessera_gb300.trees import Forest, LeafStage, lift

    leaves = lift(list(range(1, 17)))
    h = ctypes.c_void_p()

    def opened(**fields):
        spec = N.TreeC()
        spec.kind, spec.s, spec.height = 0, 0, 4
        spec.leaves = leaves.ctypes.data
        for k, v in fields.items():
            setattr(spec, k, v)
        arr = (N.TreeC * 1)(spec)
        return N.lib().tg_leaf_stage_open(dev.handle, arr, 1, 0, ctypes.byref(h))

    assert opened(kind=2) < 0
    assert opened(s=30, height=12) < 0  # 42 variables
    assert opened(kind=1, s=1, denominators=leaves.ctypes.data) < 0
    assert opened(kind=1, base_leaves=1, denominators=leaves.ctypes.data) < 0
    assert opened(leaves=None) < 0
    assert opened(kind=1, denominators=None) < 0
    ctx = SessionContext("tessera-protocol/1", Mode.NON_INTERACTIVE, "test-small/1", bytes(32), bytes(16))
    t = Transcript(ctx)
    with LeafStage([Forest(0, leaves)], dev) as st:
        st.prove(t)
        before = (t.state, t.counter)
        with pytest.raises(N.TesseraError):
            st.prove_level(t)
        assert (t.state, t.counter) == before


@pytest.fixture(scope="module")
def dev_q1():
    from tessera_gb300.device import Device

    d = Device(0, tree_sum_q1=True)
    yield d
    d.close()


def test_summed_q1_gives_the_golden_proofs(dev_q1):
    """With every round summing q(1) on the device (the path a point coordinate of 0 takes, else
    out of reach: the points are transcript challenges) instead of deriving it from the round's
    claim, the golden tree, forest and LogUp batches come out the same, level by level."""
    for base, on_device in LEAF_FORMS[:2]:
        test_tree_batches(dev_q1, base, on_device)
        test_forest_batches(dev_q1, base, on_device)
    test_logup_leaf_stages(dev_q1)


@pytest.mark.parametrize("kind", ["unit17", "fraction14", "forest6x14", "forest_fp2_4x12"])
def test_summed_q1_matches_derived_in_launched_rounds(dev, dev_q1, kind):
    """Trees large enough for launched rounds of every kind and mode (numerators of 1, fractions,
    prime-field and Fp2 products) before each level's tail: the proof with q(1) summed equals the
    proof with q(1) derived, every record, the final claim and the transcript state."""
    import torch

    from tessera_gb300.hash import Mode, SessionContext, Transcript
    from tessera_gb300.trees import Forest, LeafStage, generated_fraction, lift
    from tessera_gb300.workloads import fill_counter

    ctx = SessionContext("tessera-protocol/1", Mode.NON_INTERACTIVE, "test-small/1", bytes([3]) * 32, bytes([5]) * 16)
    if kind.startswith("forest"):
        s, h = (6, 14) if kind == "forest6x14" else (4, 12)
        leaves = fill_counter(torch.empty(1 << (s + h), dtype=torch.int64, device="cuda"), 1 << 61, dev)
        host = leaves.cpu().numpy().view(np.uint64)

    def prove(d):
        if kind.startswith("forest"):
            tree = Forest(s, leaves, True) if kind == "forest6x14" else Forest(s, lift(host))
        else:
            h = 17 if kind == "unit17" else 14
            tree = generated_fraction(h, 1000, 2000000, None if kind == "unit17" else 77, (123456789, 987654321),
                                      (55555, 4444444), d)
        t = Transcript(ctx)
        with LeafStage([tree], d) as st:
            recs = st.prove(t)
            return ([(r.rounds, r.challenges, r.claims, r.final_evals, r.rho) for r in recs], st.claim(0),
                    t.state.hex(), t.counter)

    assert prove(dev) == prove(dev_q1)


@pytest.mark.parametrize("unit,h", [(True, 0), (False, 1), (True, 2), (False, 3), (True, 9), (False, 12), (True, 14)])
def test_deferred_generated_leaves_match(dev, unit, h):
    """Leaves generated by the leaf stage itself, in the same pass as the two levels above them,
    are the generator's leaves, and the proof equals the one over leaves generated beforehand."""
    from tessera_gb300.hash import Mode, SessionContext, Transcript
    from tessera_gb300.trees import LeafStage, generated_fraction

    ctx = SessionContext("tessera-protocol/1", Mode.NON_INTERACTIVE, "test-small/1", bytes([1]) * 32, bytes([2]) * 16)
    args = (h, 31, 4000, None if unit else 900, (987654321, 123), (77, 1 << 40))
    runs = []
    for deferred in (False, True):
        tree = generated_fraction(*args, dev, deferred=deferred)
        t = Transcript(ctx)
        with LeafStage([tree], dev) as st:
            recs = st.prove(t)
            proof = ([(r.rounds, r.challenges, r.claims, r.final_evals, r.rho) for r in recs], st.claim(0), t.state.hex())
        leaves = (tree.denominators.cpu().numpy().copy(), None if unit else tree.numerators.cpu().numpy().copy())
        runs.append((proof, leaves))
    assert runs[0][0] == runs[1][0]
    assert np.array_equal(runs[0][1][0], runs[1][1][0])
    if not unit:
        assert np.array_equal(runs[0][1][1], runs[1][1][1])


def test_generated_leaves_refusals(dev):
    """A generator needs device buffers (16-byte aligned, numerators exactly when not unit) and a
    fraction tree; anything else is refused before any work."""
    import ctypes

    import torch

    from tessera_gb300 import _native as N
    from tessera_gb300.trees import LeafGen, LeafStage

    g = LeafGen(1, 2, None, (3, 4), (5, 6))
    den = torch.empty(2 * 8, dtype=torch.int64, device="cuda")
    num = torch.empty(2 * 8, dtype=torch.int64, device="cuda")
    from tessera_gb300.trees import Fraction

    with pytest.raises(N.InvalidInput):  # unit generator with a numerators buffer
        LeafStage([Fraction(den, num, gen=g)], dev)
    with pytest.raises(N.InvalidInput):  # generated numerators without a buffer
        LeafStage([Fraction(den, None, gen=LeafGen(1, 2, 3, (3, 4), (5, 6)))], dev)
    with pytest.raises(N.InvalidInput):  # not canonical
        LeafStage([Fraction(den, None, gen=LeafGen(1, 2, None, (P, 4), (5, 6)))], dev)
    arr = (N.TreeC * 1)()
    gc = N.LeafGenC(1, 2, 0, 1, (ctypes.c_uint64 * 2)(3, 4), (ctypes.c_uint64 * 2)(5, 6))
    host = np.zeros(16, dtype=np.uint64)
    arr[0].kind, arr[0].height, arr[0].denominators, arr[0].gen = 1, 3, host.ctypes.data, ctypes.addressof(gc)
    h = ctypes.c_void_p()
    with pytest.raises(N.InvalidInput):  # host memory
        N.call("tg_leaf_stage_open", dev.handle, arr, 1, 0, ctypes.byref(h))
    arr[0].kind, arr[0].leaves = 0, host.ctypes.data
    with pytest.raises(N.InvalidInput):  # a forest
        N.call("tg_leaf_stage_open", dev.handle, arr, 1, 1, ctypes.byref(h))


def _random_fp2(rng, n):
    return [(int(a), int(b)) for a, b in zip(rng.integers(0, P, size=n, dtype=np.uint64),
                                             rng.integers(0, P, size=n, dtype=np.uint64))]


@pytest.mark.parametrize("seed", [11, 12, 13])
def test_random_stages_match_the_oracle(dev, seed):
    """Random mixed stages beyond the golden shapes — forests of several root counts and heights,
    fraction trees with and without numerators of 1, trees joining at different levels — proven on
    the device and by the oracle's restatement of the tree-level prover: every level record, the
    claims each tree carries and the transcript state agree."""
    from golden_data import context_tce
    from oracle import trees as OT
    from oracle.oracle import OracleTranscript
    from tessera_gb300.trees import Forest, Fraction, LeafStage

    rng = np.random.default_rng(seed)
    shapes = [("forest", 2, 3), ("fraction", 0, 4), ("unit", 0, 2), ("forest", 0, 5), ("forest", 3, 1)]
    gpu_trees, o_trees = [], []
    for kind, s, h in shapes[: 3 + seed % 3]:
        if kind == "forest":
            lv = _random_fp2(rng, 1 << (s + h))
            gpu_trees.append(Forest(s, words(lv)))
            o_trees.append(OT.OTree(0, s, leaves=lv))
        else:
            den = _random_fp2(rng, 1 << h)
            num_ = None if kind == "unit" else _random_fp2(rng, 1 << h)
            gpu_trees.append(Fraction(words(den), None if num_ is None else words(num_)))
            o_trees.append(OT.OTree(1, 0, numerators=num_, denominators=den))
    ctx = {"protocol": "tessera-protocol/1", "mode": "NonInteractive", "params": "test-small/1",
           "statement_digest": "65" * 32, "session_id": "%032x" % seed}
    tce = context_tce(ctx)
    from tessera_gb300.hash import Transcript

    t_gpu, t_or = Transcript(tce), OracleTranscript(tce)
    ost = OT.OStage(o_trees)
    with LeafStage(gpu_trees, dev) as st:
        assert st.height == ost.H
        for _ in range(st.height):
            rec, want = st.prove_level(t_gpu), ost.prove_level(t_or)
            assert rec.root_challenges == want["root_challenges"]
            assert rec.gamma == want["gamma"] and rec.lambda_ == want["lambda"]
            assert rec.rounds == want["rounds"] and rec.challenges == want["challenges"]
            assert rec.claims == want["claims"] and rec.final_evals == want["final_evals"]
            assert rec.rho == want["rho"] and rec.present == want["present"]
            assert rec.state.hex() == want["state"] and rec.counter == want["counter"]
            for k in rec.present:
                point, claim, _ = st.claim(k)
                assert (point, claim) == ost.claim(k)
