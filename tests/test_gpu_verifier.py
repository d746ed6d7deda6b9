"""GPU proofs through the restated independent verifier (oracle/verifier.py).

Byte equality with the oracle prover shows the GPU proves what the reference's prover proves;
these tests show that a verifier accepts it: the sumchecks of the plain (32 x 2^14, Σ f·g over
2^14) and large (256 x 2^20, Σ f·g·h over 2^22) workloads with their final evaluations checked
against the tables' multilinear extensions; the commitments of both workloads answering drawn
column queries with a canonical multiproof from the device's Merkle nodes; every advice opening of
the reference's vectors assembled from the GPU's BlockSink, merge, Merkle tree and ColumnSink; and
the LogUp leaf stages, forests and generated trees level by level, the cheating batches rejected
with the reference's reasons."""
import numpy as np
import pytest

from golden_data import context_tce, fp2s, load, num
from oracle import oracle as O
from oracle import verifier as V
from oracle.verifier import Reject

pytestmark = pytest.mark.gpu
P = V.P
THREADS = O.threads_available()


@pytest.fixture(scope="module")
def dev():
    from tessera_gb300.device import default_device

    return default_device()


def bench_context():
    from tessera_gb300.hash import Mode, SessionContext

    return SessionContext("tessera-protocol/1", Mode.NON_INTERACTIVE, "test-small/1", bytes([0x65]) * 32, bytes([0x65]) * 16)


def fp_sum(words: np.ndarray) -> int:
    """Σ words mod p, exactly (32-bit halves summed in 64-bit lanes)."""
    w = words.astype(np.uint64)
    lo = int(np.sum(w & np.uint64(0xFFFFFFFF), dtype=np.uint64))
    hi = int(np.sum(w >> np.uint64(32), dtype=np.uint64))
    return (lo + (hi << 32)) % P


@pytest.mark.parametrize("log_n,degree", [(14, 2), (22, 3)])
def test_gpu_sumcheck_is_accepted(dev, log_n, degree):
    """The GPU's proof of Σ Π tables over 2^log_n prime-field entries passes verify_batch on a
    fresh transcript (γ, point and final state equal to the prover's), its final evaluations are
    the tables' MLEs at the point, and a changed message or evaluation is rejected."""
    from tessera_gb300.hash import Transcript
    from tessera_gb300.sumcheck import Instance, Protocol, Table, prove_batch

    tabs = [O.splitmix(0x00650010 + 7 * log_n + i, 1 << log_n) for i in range(degree)]
    prod = tabs[0]
    for tb in tabs[1:]:
        prod = O.fp_vec("mul", prod, tb)
    claim = (fp_sum(prod), 0)
    t = Transcript(bench_context())
    pb = prove_batch(t, Protocol.ONE, "stage/0", degree, [Instance([Table.base(x) for x in tabs])], device=dev)
    rounds, evals = pb.proof.rounds, pb.proof.final_evals
    tv = O.OracleTranscript(bench_context().tce())
    gamma, point = V.verify_batch(tv, "stage/0", degree, [(claim, log_n, degree)], rounds, evals, V.product_relation)
    assert gamma == pb.gamma and point == pb.point
    assert (tv.state, tv.counter) == (t.state, t.counter)
    assert evals == [O.mle(tb, point) for tb in tabs]
    bad = [list(m) for m in rounds]
    bad[log_n // 2][1] = V.add(bad[log_n // 2][1], (1, 0))
    with pytest.raises(Reject):
        V.verify_batch(O.OracleTranscript(bench_context().tce()), "stage/0", degree, [(claim, log_n, degree)], bad,
                       evals, V.product_relation)
    with pytest.raises(Reject):
        V.verify_batch(O.OracleTranscript(bench_context().tce()), "stage/0", degree, [(V.add(claim, (1, 0)), log_n, degree)],
                       rounds, evals, V.product_relation)


@pytest.mark.parametrize("npolys,log_k,log_r", [(32, 14, 2), (256, 20, 1)])
def test_gpu_commitment_answers_are_accepted(dev, npolys, log_k, log_r):
    """The commitment of the plain and the large workload (B = 32) answers 64 column queries
    drawn from a transcript that absorbed its root: the queried columns' symbols from the device
    codewords, the canonical multiproof from the device's Merkle nodes. The verifier recomputes
    each leaf from the symbols (the column's chain) and the root from the multiproof; a changed
    symbol or sibling is rejected."""
    import ctypes

    import torch

    from tessera_gb300 import _native as N
    from tessera_gb300.hash import Transcript
    from tessera_gb300.workloads import fill_device

    B = 32
    n = 1 << (log_k + log_r)
    cid = bytes([0x65]) * 32
    rows = fill_device(torch.empty(npolys << log_k, dtype=torch.int64, device="cuda"), 0x00650020 + log_k, dev)
    cw = torch.empty(npolys * n, dtype=torch.int64, device="cuda")
    nodes = torch.empty((2 * n - 1) * 32, dtype=torch.uint8, device="cuda")
    root = ctypes.create_string_buffer(32)
    torch.cuda.synchronize()
    N.call("tg_commit_unmasked_dev", dev.handle, log_k, log_r, B, (ctypes.c_uint8 * 32)(*cid),
           ctypes.c_void_p(rows.data_ptr()), npolys, ctypes.c_void_p(cw.data_ptr()), ctypes.c_void_p(nodes.data_ptr()),
           root, None)
    dev.sync()
    t = Transcript(bench_context())
    t.absorb("commit/root", root.raw)
    queries = t.challenge_indices("commit/queries", log_k + log_r, 64)
    distinct = sorted(set(queries))
    idx = torch.tensor(distinct, dtype=torch.int64, device="cuda")
    cols = cw.view(npolys, n)[:, idx].cpu().numpy().view(np.uint64).T  # distinct x npolys
    del rows, cw
    nd = nodes.cpu().numpy().reshape(-1, 32)
    siblings = V.canonical_multiproof(nd, n, distinct)
    leaves = [(j, V.column_digest(cid, j, list(cols[q]), B)) for q, j in enumerate(distinct)]
    V.verify_multiproof(root.raw, n, leaves, siblings)
    bad = [list(c) for c in cols]
    bad[0][npolys - 1] = (int(bad[0][npolys - 1]) + 1) % P
    with pytest.raises(Reject):
        V.verify_multiproof(root.raw, n, [(j, V.column_digest(cid, j, bad[q], B)) for q, j in enumerate(distinct)],
                            siblings)
    with pytest.raises(Reject):
        V.verify_multiproof(root.raw, n, leaves, [siblings[1], siblings[0]] + siblings[2:])


def _witness(op):
    k, PA = 1 << op["log2_k"], op["mask_coeffs"]
    rows = np.array([[num(x) for x in r] for r in op["witness"]["rows"]], dtype=np.uint64).reshape(-1, k)
    masks = np.array([[num(x) for x in m] for m in op["witness"]["masks"]], dtype=np.uint64).reshape(-1, PA)
    return rows, masks


def gpu_opening(dev, op):
    """An advice opening assembled from the GPU: each segment's chains through the BlockSink,
    the merged leaves and root, the Merkle tree, the queried columns and P4's combined rows u_g
    through the ColumnSink; the combined masks M_g are the host's part, as in the reference."""
    from tessera_gb300.hash import MerkleTree
    from tessera_gb300.pcs import AdviceSink, ColumnSink, CommitmentParams, RowEncoder, merge_segments

    lk, lr, PA, B = op["log2_k"], op["log2_inv_rate"], op["mask_coeffs"], op["row_block"]
    k, n = 1 << lk, 1 << (lk + lr)
    rows, masks = _witness(op)
    cid = bytes.fromhex(op["commitment_id"])
    parts, at = [], 0
    for seg in op["segments"]:
        sink = AdviceSink(CommitmentParams(lk, lr, PA, B, cid), device=dev)
        for b in range(0, len(seg), B):
            e = min(len(seg), b + B)
            sink.absorb(rows[at + b:at + e], masks[at + b:at + e])
        parts.append(sink.finish())
        sink.close()
        at += len(seg)
    adv = merge_segments(parts, device=dev)
    tree = MerkleTree(adv.leaves, device=dev)
    distinct = sorted(set(op["queries"]))
    coeffs = V.row_coefficients(op)
    sink = ColumnSink(RowEncoder(k, lr, PA, device=dev), B, distinct, device=dev)
    got = []
    for b in range(0, len(rows), B):
        e = min(len(rows), b + B)
        got.append(sink.select_combining(rows[b:e], masks[b:e], [c[b:e] for c in coeffs]))
    u = sink.combined(np.zeros((len(coeffs), k, 2), dtype=np.uint64))
    sink.close()
    cols = np.concatenate(got).T  # distinct x rows
    combined = []
    for g, cs in enumerate(coeffs):
        m = [V.ZERO] * PA
        for ri, c in enumerate(cs):
            m = [V.add(m[i], V.T.scale(c, int(masks[ri, i]))) for i in range(PA)]
        combined.append({"u": [[hex(int(a)), hex(int(b))] for a, b in u[g]], "mask": [[hex(a), hex(b)] for a, b in m]})
    assembled = dict(op)
    assembled.update(root=adv.root.hex(), combined=combined, columns=[[hex(int(x)) for x in c] for c in cols],
                     siblings=[s.hex() for s in V.canonical_multiproof(tree.nodes(), n, distinct)])
    return assembled


def test_gpu_openings_match_and_are_accepted(dev):
    """Every honest opening of the reference's vectors, assembled from the GPU, equals the
    vectors' root, combined rows, columns and multiproof value for value and passes the verifier."""
    for op in load("opening")["openings"]:
        got = gpu_opening(dev, op)
        assert got["root"] == op["root"], op["name"]
        for c, want in zip(got["combined"], op["combined"]):
            assert fp2s(c["u"]) == fp2s(want["u"]) and fp2s(c["mask"]) == fp2s(want["mask"]), op["name"]
        assert [[num(x) for x in c] for c in got["columns"]] == [[num(x) for x in c] for c in op["columns"]], op["name"]
        assert got["siblings"] == op["siblings"], op["name"]
        V.verify_opening(got)


def _log_records(recs):
    return [{"rounds": r.rounds, "final_evals": r.final_evals} for r in recs]


def test_gpu_logup_stages_are_verified(dev):
    """The GPU proves every LogUp batch whose prover the vectors describe; the verifier accepts
    the honest ones (its transcript ending in the prover's state) and rejects the cheats with the
    reference's reason and check."""
    from test_gpu_trees import forest_of, logup_trees, mle, transcript
    from test_oracle_verifier import logup_schedule

    from tessera_gb300.trees import LeafStage

    seen = {"accept": 0, "reject": 0}
    for b in load("trees")["logup_batches"]:
        exp = b["expected"]
        if exp != "accept" and exp["check"] != "roots" and not exp["check"].startswith("level"):
            continue
        t = transcript(b["context"])
        alpha, beta = t.challenge_fp2("logup/alpha"), t.challenge_fp2("logup/beta")
        built = [logup_trees(alpha, beta, inst) for inst in b["instances"]]
        sent = fp2s(b["roots"])
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
            recs = st.prove(t)
            place = {(e["kind"], e["index"]): k for k, e in enumerate(b["trees"])}
            values = [mle(built[i][2], st.claim(place[("lookup", i)])[0])
                      for i, inst in enumerate(b["instances"]) if inst["has_values"]]
        t.absorb_fp2s("logup/values", values)
        sched, tables = logup_schedule(b)
        tv = O.OracleTranscript(context_tce(b["context"]))
        if exp == "accept":
            V.verify_leaf_stage(tv, sched, _log_records(recs), roots=sent, values=values, tables=tables)
            assert (tv.state, tv.counter) == (t.state, t.counter), b["name"]
            seen["accept"] += 1
        else:
            with pytest.raises(Reject) as e:
                V.verify_leaf_stage(tv, sched, _log_records(recs), roots=sent, values=values, tables=tables)
            assert (e.value.reason, e.value.detail["check"]) == (exp["reason"], exp["check"]), b["name"]
            seen["reject"] += 1
    assert seen["accept"] >= 10 and seen["reject"] >= 5


@pytest.mark.parametrize("kind,h", [("unit", 14), ("mult", 17), ("forest", 14)])
def test_gpu_large_trees_are_verified(dev, kind, h):
    """Generated LogUp trees of heights 14 and 17 (launched rounds and the single-block tail) and a
    forest of 2^6 trees of 2^14 prime-field counter leaves: the verifier runs every level from the
    root claims to the leaf claims, ending in the prover's transcript state, and the leaf claims
    are the leaves' MLEs."""
    import torch

    from tessera_gb300.hash import Mode, SessionContext, Transcript
    from tessera_gb300.trees import Forest, LeafStage, generated_fraction
    from tessera_gb300.workloads import fill_counter

    ctx = SessionContext("tessera-protocol/1", Mode.NON_INTERACTIVE, "test-small/1", bytes(32), bytes(16))
    t = Transcript(ctx)
    if kind == "forest":
        s = 6
        leaves = fill_counter(torch.empty(1 << (s + h), dtype=torch.int64, device="cuda"), 5000, dev)
        tree = Forest(s, leaves, base=True)
    else:
        tree = generated_fraction(h, 1000, 2000000, None if kind == "unit" else 77, (123456789, 987654321),
                                  (55555, 4444444), dev)
    with LeafStage([tree], dev) as st:
        roots = st.root(0)
        recs = st.prove(t)
        point, final, _ = st.claim(0)
    if kind == "forest":
        tv = O.OracleTranscript(ctx.tce())
        rootc = [tv.challenge_fp2(f"tree/0/root/{c}") for c in range(s)]
        claim = ("product", rootc, V.T.mle(roots, rootc))
    else:
        tv = O.OracleTranscript(ctx.tce())
        claim = ("fraction", [], roots[0], roots[1])
    for level, rec in enumerate(recs):
        _, _, _, _, nxt = V.verify_level(tv, f"tree/{level}", [claim], rec.rounds, rec.final_evals)
        claim = nxt[0]
    assert (tv.state, tv.counter) == (t.state, t.counter)
    assert claim[1] == point
    if kind == "forest":
        words = leaves.cpu().numpy().view(np.uint64)
        assert claim[2] == final == O.mle(words, point)
    else:
        d = tree.denominators.cpu().numpy().view(np.uint64)
        assert (claim[2], claim[3]) == final
        assert claim[3] == O.mle(d, point, is_ext=True)
        if tree.numerators is not None:
            assert claim[2] == O.mle(tree.numerators.cpu().numpy().view(np.uint64), point, is_ext=True)
        else:
            assert claim[2] == (1, 0)
