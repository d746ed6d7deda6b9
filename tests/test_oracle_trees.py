"""CPU: the oracle's restatement of the tree-level prover (oracle/trees.py) reproduces the
reference's golden tree batches, product-forest batches and honest LogUp leaf stages level by level
— root challenges, γ, λ, round messages, challenges, the verifier's claims, final evaluations, ρ,
the transcript state and every claim carried to the next level. This pins the oracle that the GPU
tree tests can then be compared against on other inputs."""
import gzip
import json
from pathlib import Path

from golden_data import context_tce
from oracle import trees as T
from oracle.oracle import OracleTranscript

GOLD = json.load(gzip.open(Path(__file__).parent / "golden" / "trees.json.gz"))


def num(x):
    return int(x, 16)


def f2(pair):
    return (num(pair[0]), num(pair[1]))


def f2s(items):
    return [f2(p) for p in items]


def check(rec, want, stage, name):
    assert rec["prefix"] == want["prefix"], name
    assert rec["root_challenges"] == f2s(want.get("root_challenges", [])), name
    assert rec["gamma"] == f2(want["gamma"]), name
    if "lambda" in want:
        assert rec["lambda"] == (None if want["lambda"] is None else f2(want["lambda"])), name
    assert rec["rounds"] == [f2s(m) for m in want["rounds"]], name
    assert rec["challenges"] == f2s(want["challenges"]), name
    assert rec["claims"] == f2s(want["claims"]), name
    assert rec["final_evals"] == f2s(want["final_evals"]), name
    assert rec["rho"] == f2(want["rho"]), name
    assert rec["state"] == want["state"] and rec["counter"] == want["counter"], name
    key = "tree" if "tree" in want["next"][0] else "forest"
    assert [n[key] for n in want["next"]] == rec["present"], name
    for n in want["next"]:
        point, claim = stage.claim(n[key])
        assert point == f2s(n["point"]), name
        if "value" in n:
            assert claim == f2(n["value"]), name
        else:
            assert claim == (f2(n["numerator"]), f2(n["denominator"])), name


def test_oracle_tree_batches():
    for b in GOLD["tree_batches"]:
        t = OracleTranscript(context_tce(b["context"]))
        st = T.OStage([T.OTree(0, 0, leaves=[(num(x), 0) for x in tr["leaves"]]) for tr in b["trees"]])
        for k, tr in enumerate(b["trees"]):
            assert st.trees[k].root() == [(num(tr["root"]), 0)], b["name"]
        for want in b["levels"]:
            check(st.prove_level(t), want, st, b["name"])


def test_oracle_forest_batches():
    for b in GOLD["forest_batches"]:
        t = OracleTranscript(context_tce(b["context"]))
        st = T.OStage([T.OTree(0, f["rows_log"], leaves=[(num(x), 0) for x in f["leaves"]]) for f in b["forests"]])
        for k, f in enumerate(b["forests"]):
            assert st.trees[k].root() == [(num(x), 0) for x in f["roots"]], b["name"]
        for want in b["levels"]:
            check(st.prove_level(t), want, st, b["name"])


def _compress(beta, row):
    return T.add((row[0], 0), T.mul(beta, (row[1], 0)))


def test_oracle_logup_leaf_stages():
    """The honest LogUp batches (and the cheats that change only lookups, multiplicities or the
    roots message): α, β, the roots message, every level of the leaf stage and the final state."""
    checked = 0
    for b in GOLD["logup_batches"]:
        exp = b["expected"]
        kind = "accept" if exp == "accept" else ("roots" if exp.get("check") == "roots" else
                                                  "level" if str(exp.get("check", "")).startswith("level") else "other")
        if kind == "other":
            continue
        t = OracleTranscript(context_tce(b["context"]))
        alpha, beta = t.challenge_fp2("logup/alpha"), t.challenge_fp2("logup/beta")
        assert (alpha, beta) == (f2(b["alpha"]), f2(b["beta"])), b["name"]
        sent = f2s(b["roots"])
        t.absorb("logup/roots", T.tce_fp2s(sent))
        built = []
        for inst in b["instances"]:
            rows = [(num(k), num(v)) for k, v in inst["rows"]]
            tuples = [rows[j] if isinstance(j, int) else (num(j[0]), num(j[1])) for j in inst["lookups"]]
            slots = tuples + [rows[0]] * ((1 << inst["h_a"]) - len(tuples))
            table_rows = rows + [rows[0]] * ((1 << inst["h_t"]) - len(rows))
            m = [num(x) for x in inst["multiplicities"]]
            built.append(([T.sub(alpha, _compress(beta, tp)) for tp in slots],
                          [((T.P - mj) % T.P, 0) for mj in m], [T.sub(alpha, _compress(beta, r)) for r in table_rows]))
        schedule = []
        for entry in b["trees"]:
            if entry["kind"] == "forest":
                f = b["forests"][entry["index"]]
                schedule.append(T.OTree(0, f["rows_log"], leaves=[(num(x), 0) for x in f["leaves"]]))
            else:
                i = entry["index"]
                side = 0 if entry["kind"] == "lookup" else 1
                s = (sent[4 * i + 2 * side], sent[4 * i + 2 * side + 1])
                if side == 0:
                    schedule.append(T.OTree(1, 0, denominators=built[i][0], sent=s))
                else:
                    schedule.append(T.OTree(1, 0, numerators=built[i][1], denominators=built[i][2], sent=s))
        st = T.OStage(schedule)
        for want in b["levels"]:
            check(st.prove_level(t), want, st, b["name"])
        checked += 1
    assert checked >= 12
