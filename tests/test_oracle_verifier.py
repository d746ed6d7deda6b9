"""CPU: the restated verifier (oracle/verifier.py) against the reference's golden vectors.

It accepts every honest golden sumcheck stage, product-tree batch, forest batch and LogUp leaf
stage, rederiving every challenge and the transcript state; it rejects every cheating LogUp batch
with the reason, check and instance the reference records, and tampered messages; it accepts every
honest advice opening of spec/vectors/pcs/opening.json and rejects each of its rejections with
the stated reason, group and column. The oracle's P4 combination and P5 answer reproduce those
openings from their witnesses value for value. This pins the checker that the GPU tests then run
every GPU proof through."""
import numpy as np
import pytest

from golden_data import context_tce, fp2s, load, num
from oracle import oracle as O
from oracle import verifier as V
from oracle.verifier import Reject

P = V.P


def f2(pair):
    return (num(pair[0]), num(pair[1]))


def stage_proof(stage):
    return [fp2s(m) for m in stage["rounds"]], fp2s(stage["final_evals"])


def test_verify_golden_sumcheck_stages():
    gold = load("sumcheck")
    checked = 0
    for session in gold["sessions"]:
        t = O.OracleTranscript(context_tce(session["context"]))
        for st in session["stages"]:
            inst = [(f2(i["claim"]), i["vars"], i["factors"]) for i in st["instances"]]
            rounds, evals = stage_proof(st)
            gamma, point = V.verify_batch(t, st["prefix"], st["degree"], inst, rounds, evals, V.product_relation)
            assert gamma == f2(st["gamma"]) and point == fp2s(st["challenges"]), session["name"]
            assert (t.state.hex(), t.counter) == (st["state"], st["counter"]), session["name"]
            checked += 1
    assert checked == 62


def _first_stage_with_rounds():
    for session in load("sumcheck")["sessions"]:
        for k, st in enumerate(session["stages"]):
            if st["rounds"] and k == 0:
                return session, st
    raise AssertionError("no stage with rounds")


@pytest.mark.parametrize("tamper", ["round value", "final eval", "claim", "missing round", "extra round",
                                    "round length", "eval count"])
def test_verify_batch_rejects_tampered_stages(tamper):
    session, st = _first_stage_with_rounds()
    inst = [(f2(i["claim"]), i["vars"], i["factors"]) for i in st["instances"]]
    rounds, evals = stage_proof(st)
    if tamper == "round value":
        rounds[-1][0] = V.add(rounds[-1][0], (1, 0))
    elif tamper == "final eval":
        evals[0] = V.add(evals[0], (0, 1))
    elif tamper == "claim":
        inst[0] = (V.add(inst[0][0], (1, 0)),) + inst[0][1:]
    elif tamper == "missing round":
        rounds = rounds[:-1]
    elif tamper == "extra round":
        rounds = rounds + [rounds[-1]]
    elif tamper == "round length":
        rounds[0] = rounds[0] + [(0, 0)]
    else:
        evals = evals[:-1]
    t = O.OracleTranscript(context_tce(session["context"]))
    with pytest.raises(Reject) as e:
        V.verify_batch(t, st["prefix"], st["degree"], inst, rounds, evals, V.product_relation)
    assert e.value.reason == "Sumcheck"


def _levels(batch):
    return [{"rounds": [fp2s(m) for m in lv["rounds"]], "final_evals": fp2s(lv["final_evals"])} for lv in batch["levels"]]


def _log2(n):
    return n.bit_length() - 1


def test_verify_golden_tree_and_forest_batches():
    gold = load("trees")
    for b in gold["tree_batches"]:
        t = O.OracleTranscript(context_tce(b["context"]))
        sched = [{"kind": "forest", "s": 0, "h": _log2(len(tr["leaves"])), "roots": [(num(tr["root"]), 0)]}
                 for tr in b["trees"]]
        held, _ = V.verify_leaf_stage(t, sched, _levels(b))
        assert (t.state.hex(), t.counter) == (b["levels"][-1]["state"], b["levels"][-1]["counter"]), b["name"]
        for k, tr in enumerate(b["trees"]):
            _, point, value = held[k]
            assert value == V.T.mle([(num(x), 0) for x in tr["leaves"]], point), b["name"]  # the leaf claim
    for b in gold["forest_batches"]:
        t = O.OracleTranscript(context_tce(b["context"]))
        sched = [{"kind": "forest", "s": f["rows_log"], "h": f["height"], "roots": [(num(x), 0) for x in f["roots"]]}
                 for f in b["forests"]]
        held, _ = V.verify_leaf_stage(t, sched, _levels(b))
        assert (t.state.hex(), t.counter) == (b["levels"][-1]["state"], b["levels"][-1]["counter"]), b["name"]
        for k, f in enumerate(b["forests"]):
            _, point, value = held[k]
            assert value == V.T.mle([(num(x), 0) for x in f["leaves"]], point), b["name"]


def logup_schedule(b):
    sched = []
    for entry in b["trees"]:
        if entry["kind"] == "forest":
            f = b["forests"][entry["index"]]
            sched.append({"kind": "forest", "s": f["rows_log"], "h": f["height"], "roots": [(num(x), 0) for x in f["roots"]]})
        else:
            inst = b["instances"][entry["index"]]
            sched.append({"kind": entry["kind"], "instance": entry["index"],
                          "h": inst["h_a"] if entry["kind"] == "lookup" else inst["h_t"]})
    tables = [([(num(k), num(v)) for k, v in inst["rows"]], inst["has_values"], inst["h_t"]) for inst in b["instances"]]
    return sched, tables


def verify_logup_batch(b, levels=None, roots=None, values=None):
    t = O.OracleTranscript(context_tce(b["context"]))
    sched, tables = logup_schedule(b)
    return t, V.verify_leaf_stage(t, sched, levels if levels is not None else _levels(b),
                                  roots=roots if roots is not None else fp2s(b["roots"]),
                                  values=values if values is not None else fp2s(b["values"]), tables=tables)


def test_verify_golden_logup_batches():
    """Honest batches are accepted with the recorded final state and leaf checks; every cheating
    batch is rejected with the reference's reason and check (and instance, for LogUp's own checks)."""
    accepted = rejected = 0
    for b in load("trees")["logup_batches"]:
        exp = b["expected"]
        if exp == "accept":
            t, (_, claims) = verify_logup_batch(b)
            assert (t.state.hex(), t.counter) == (b["state"], b["counter"]), b["name"]
            for c, want in zip(claims, b["leaf_checks"]):
                assert c["key"][1] == f2(want["lookup"]["key"]), b["name"]
                assert c["multiplicity"][1] == f2(want["table"]["multiplicity"]), b["name"]
            accepted += 1
            continue
        with pytest.raises(Reject) as e:
            verify_logup_batch(b)
        r = e.value
        assert (r.reason, r.detail.get("check")) == (exp["reason"], exp["check"]), (b["name"], r)
        if exp["reason"] == "Lookup":
            assert r.detail.get("instance") == exp["instance"], b["name"]
        rejected += 1
    assert accepted >= 10 and rejected >= 10


def test_verify_logup_rejects_tampered_messages():
    b = next(x for x in load("trees")["logup_batches"] if x["expected"] == "accept" and len(x["levels"]) >= 2)
    roots = fp2s(b["roots"])
    bad = list(roots)
    bad[0] = V.add(bad[0], (1, 0))
    with pytest.raises(Reject) as e:
        verify_logup_batch(b, roots=bad)
    assert e.value.reason == "Lookup" and e.value.detail["check"] == "roots"
    levels = _levels(b)
    levels[1]["final_evals"][0] = V.add(levels[1]["final_evals"][0], (0, 1))
    with pytest.raises(Reject) as e:
        verify_logup_batch(b, levels=levels)
    assert (e.value.reason, e.value.detail["check"]) == ("Sumcheck", "level 1")
    values = fp2s(b["values"])
    with pytest.raises(Reject) as e:
        verify_logup_batch(b, values=values + [(1, 0)])
    assert (e.value.reason, e.value.detail["check"]) == ("Lookup", "values length")
    if values:
        # a changed value passes the leaf checks but moves the key claim the lookups must meet later
        _, (_, honest) = verify_logup_batch(b)
        values[0] = V.add(values[0], (1, 0))
        _, (_, moved) = verify_logup_batch(b, values=values)
        assert moved[0]["key"] != honest[0]["key"]


def test_verify_golden_openings():
    gold = load("opening")
    for op in gold["openings"]:
        V.verify_opening(op)
    for rj in gold["rejections"]:
        with pytest.raises(Reject) as e:
            V.verify_opening(rj["opening"])
        r = e.value
        assert r.reason == rj["reason"], rj["name"]
        assert r.detail.get("group") == rj["group"] and r.detail.get("column") == rj["column"], rj["name"]


def _witness(op):
    k, PA = 1 << op["log2_k"], op["mask_coeffs"]
    rows = np.array([[num(x) for x in r] for r in op["witness"]["rows"]], dtype=np.uint64).reshape(-1, k)
    masks = np.array([[num(x) for x in m] for m in op["witness"]["masks"]], dtype=np.uint64).reshape(-1, PA)
    return rows, masks


def oracle_opening(op):
    """The oracle prover's opening from the witness and public inputs: codewords (masked
    encoding), per-segment chains merged into leaves, the Merkle tree, P4's combined rows
    u_g = Σ_row c_g(row)·A_row and M_g = Σ_row c_g(row)·m_row, and P5's distinct columns with
    their canonical multiproof."""
    lk, lr, PA = op["log2_k"], op["log2_inv_rate"], op["mask_coeffs"]
    n = 1 << (lk + lr)
    rows, masks = _witness(op)
    cw = O.encode_rows(rows, lk, lr, masks=masks, mask_coeffs=PA).reshape(len(rows), n)
    cid = bytes.fromhex(op["commitment_id"])
    segs, at = [], 0
    for seg in op["segments"]:
        segs.append(O.column_chains(cid, cw[at:at + len(seg)].reshape(-1), n, op["row_block"]))
        at += len(seg)
    leaves, root = O.merge_segments(np.stack(segs))
    nodes = O.merkle_tree(leaves)
    coeffs = V.row_coefficients(op)
    combined = []
    for cs in coeffs:
        u = [V.ZERO] * rows.shape[1]
        m = [V.ZERO] * PA
        for ri, c in enumerate(cs):
            u = [V.add(u[i], V.T.scale(c, int(rows[ri, i]))) for i in range(len(u))]
            m = [V.add(m[i], V.T.scale(c, int(masks[ri, i]))) for i in range(PA)]
        combined.append((u, m))
    distinct = sorted(set(op["queries"]))
    columns = [[int(cw[r, j]) for r in range(len(rows))] for j in distinct]
    siblings = V.canonical_multiproof(nodes, n, distinct)
    return root, combined, columns, siblings


def test_oracle_reproduces_golden_openings():
    for op in load("opening")["openings"]:
        root, combined, columns, siblings = oracle_opening(op)
        assert root.hex() == op["root"], op["name"]
        for (u, m), want in zip(combined, op["combined"]):
            assert u == fp2s(want["u"]) and m == fp2s(want["mask"]), op["name"]
        assert columns == [[num(x) for x in c] for c in op["columns"]], op["name"]
        assert [s.hex() for s in siblings] == op["siblings"], op["name"]
