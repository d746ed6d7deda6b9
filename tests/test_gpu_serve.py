"""The proof server (continuous batching): each served proof is byte-identical to the same proof
made alone through the plain entry points — whether the requests arrive all at once, one at a
time, at random moments from another thread, or under an HBM budget that admits one at a time —
and small proofs also match the CPU oracle."""
import random
import threading
import time

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dev():
    from tessera_gb300.device import default_device

    return default_device()


def ctx(i):
    from tessera_gb300.hash import Mode, SessionContext

    return SessionContext("tessera-protocol/1", Mode.NON_INTERACTIVE, "test-small/1", bytes([0x65]) * 32,
                          i.to_bytes(16, "little"))


def requests(count, seed=5, max_log_k=13, max_vars=13):
    from tessera_gb300.hash import Transcript
    from tessera_gb300.pcs import CommitmentParams
    from tessera_gb300.serve import ProofRequest
    from tessera_gb300.workloads import splitmix_words

    rs = random.Random(seed)
    out = []
    for i in range(count):
        log_k = rs.randint(4, max_log_k)
        polys = rs.choice([1, 3, 8, 32])
        log_r = rs.choice([1, 2])
        vars_ = rs.randint(1, max_vars)
        degree = rs.choice([1, 2, 3])
        ntab = rs.randint(1, degree)
        cid = bytes(rs.randrange(256) for _ in range(32))
        rows = splitmix_words(1000 + i, polys << log_k)
        tabs = [splitmix_words(5000 + 10 * i + k, 1 << vars_) for k in range(ntab)]
        out.append(ProofRequest(CommitmentParams(log_k, log_r, 0, rs.choice([1, 4, 32]), cid), rows, degree, tabs,
                                Transcript(ctx(i)), f"serve/{i}"))
    return out


def test_served_equals_plain_all_at_once(dev):
    from tessera_gb300.serve import ProofServer, prove_plain

    reqs = requests(24)
    plain = [prove_plain(r, dev) for r in reqs]
    with ProofServer(dev, slots=8) as srv:
        tickets = [srv.submit(r) for r in reqs]
        served = [srv.wait(t) for t in tickets]
        st = srv.stats()
    assert st["completed"] == 24 and st["peak_inflight"] >= 2
    for i, (a, b) in enumerate(zip(served, plain)):
        assert a.same_proof(b), i
        assert a.latency_ms >= a.queued_ms >= 0


def test_served_one_at_a_time_and_random_arrivals(dev):
    from tessera_gb300.serve import ProofServer, prove_plain

    reqs = requests(16, seed=9)
    plain = [prove_plain(r, dev) for r in reqs]
    with ProofServer(dev, slots=4) as srv:
        alone = [srv.wait(srv.submit(r)) for r in reqs]
    tickets = [None] * len(reqs)
    with ProofServer(dev, slots=4) as srv:
        def producer():
            rs = random.Random(3)
            for i, r in enumerate(reqs):
                tickets[i] = srv.submit(r)
                time.sleep(rs.random() * 0.004)

        th = threading.Thread(target=producer)
        th.start()
        th.join()
        mixed = [srv.wait(t) for t in tickets]
    for i in range(len(reqs)):
        assert alone[i].same_proof(plain[i]) and mixed[i].same_proof(plain[i]), i


def test_budget_admits_one_at_a_time(dev):
    """With a budget below any two requests' footprints, requests run one after another and the
    proofs are unchanged."""
    from tessera_gb300.serve import ProofServer, prove_plain

    reqs = requests(6, seed=11, max_log_k=12, max_vars=12)
    plain = [prove_plain(r, dev) for r in reqs]
    with ProofServer(dev, hbm_budget_bytes=1, slots=8) as srv:
        served = [srv.wait(t) for t in [srv.submit(r) for r in reqs]]
        st = srv.stats()
    assert st["peak_inflight"] == 1
    assert all(a.same_proof(b) for a, b in zip(served, plain))


def test_served_vs_oracle(dev):
    from tessera_gb300.serve import ProofServer

    reqs = requests(4, seed=13, max_log_k=10, max_vars=10)
    with ProofServer(dev, slots=4) as srv:
        served = [srv.wait(t) for t in [srv.submit(r) for r in reqs]]
    for i, (r, s) in enumerate(zip(reqs, served)):
        p = r.params
        _, _, root = O.commit_unmasked(r.rows, p.log2_k, p.log2_inv_rate, p.row_block, p.commitment_id,
                                       threads=O.threads_available(), keep_codewords=False)
        assert s.root == root
        ot = O.OracleTranscript(ctx(i).tce())
        ot.absorb(r.prefix + "/root", root)
        g, rounds, chal, evals = O.prove_batch(ot, r.prefix, r.degree, [[(x, False, False) for x in r.tables]])
        assert (s.gamma, s.rounds, s.challenges, s.final_evals) == (g, rounds, chal, evals)
        assert (s.state, s.counter) == (ot.state, ot.counter)


def test_submit_refusals(dev):
    from tessera_gb300 import _native as N
    from tessera_gb300.serve import ProofServer

    good = requests(1)[0]
    with ProofServer(dev, slots=2) as srv:
        for field, value in (("degree", 0), ("degree", 8), ("tables", [])):
            bad = requests(1)[0]
            setattr(bad, field, value)
            with pytest.raises(N.TesseraError):
                srv.submit(bad)
        assert srv.wait(srv.submit(good)).root


def test_served_opening_rounds_equal_plain_and_verify(dev):
    """Requests with an opening round: the query indices, the queried columns read from the
    device-resident codewords and the multiproof read from the resident Merkle nodes equal the
    plain path's (which answers from tg_commit_unmasked_dev's buffers), in a mix with requests
    that have no opening round and alone; the restated verifier accepts every answer (leaves
    recomputed from the columns' chains, the root from the multiproof) and rejects a changed
    symbol."""
    from oracle import verifier as V
    from tessera_gb300.serve import ProofServer, prove_plain

    reqs = requests(20, seed=17)
    for i, r in enumerate(reqs):
        r.queries = [0, 1, 7, 32][i % 4]
    plain = [prove_plain(r, dev) for r in reqs]
    with ProofServer(dev, slots=6) as srv:
        served = [srv.wait(t) for t in [srv.submit(r) for r in reqs]]
    with ProofServer(dev, slots=1) as srv:
        alone = [srv.wait(srv.submit(r)) for r in reqs]
    for i, (r, a, b, c) in enumerate(zip(reqs, served, plain, alone)):
        assert a.same_proof(b) and c.same_proof(b), i
        if not r.queries:
            assert a.query_indices is None
            continue
        p = r.params
        n = 1 << (p.log2_k + p.log2_inv_rate)
        distinct = sorted(set(a.query_indices))
        assert len(a.query_indices) == r.queries and a.columns.shape == (len(distinct), len(r.rows) >> p.log2_k)
        leaves = [(j, V.column_digest(p.commitment_id, j, list(a.columns[q]), p.row_block))
                  for q, j in enumerate(distinct)]
        V.verify_multiproof(a.root, n, leaves, a.siblings)
        bad = [list(col) for col in a.columns]
        bad[-1][0] = (int(bad[-1][0]) + 1) % O.P
        with pytest.raises(V.Reject):
            V.verify_multiproof(a.root, n, [(j, V.column_digest(p.commitment_id, j, bad[q], p.row_block))
                                            for q, j in enumerate(distinct)], a.siblings)


def test_opening_round_refusals(dev):
    from tessera_gb300 import _native as N
    from tessera_gb300.serve import ProofServer

    big = requests(1, seed=19)[0]
    big.queries = 1 << 20  # far beyond the answer's staging
    with ProofServer(dev, slots=2) as srv:
        with pytest.raises(N.TesseraError):
            srv.submit(big)
