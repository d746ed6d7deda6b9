"""The batched pattern on the GPU: many independent sumchecks proved together (one fused launch
per round for all of them) and many commitments committed together (on several streams, or
replayed from a captured CUDA graph) give, byte for byte, what one-at-a-time calls give — checked
against the reference's golden sessions, the CPU oracle and the plain per-job path, on the
batched workload's uneven shapes."""
import numpy as np
import pytest

from golden_data import context_tce, fp2s, load, num, stage_tables
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dev():
    from tessera_gb300.device import default_device

    return default_device()


def ctx(session_id: bytes):
    from tessera_gb300.hash import Mode, SessionContext

    return SessionContext("tessera-protocol/1", Mode.NON_INTERACTIVE, "test-small/1", bytes([0x65]) * 32, session_id)


def test_prove_many_golden_sessions(dev):
    """The reference's 9 golden sessions advance together: call k proves stage k of every session
    that has one, each on its session's transcript; all 62 stages match the golden vectors."""
    from tessera_gb300.hash import Transcript
    from tessera_gb300.sumcheck import Instance, Prefix, Protocol, Table, prove_many

    v = load("sumcheck")
    seed = num(v["seed"])
    sessions = v["sessions"]
    ts = [Transcript(context_tce(s["context"])) for s in sessions]
    count = 0
    for k in range(max(len(s["stages"]) for s in sessions)):
        live = [i for i, s in enumerate(sessions) if k < len(s["stages"])]
        jobs = []
        for i in live:
            st = sessions[i]["stages"][k]
            insts = [Instance([Table.ext(tb) for tb in inst]) for inst in stage_tables(seed, st)]
            jobs.append((ts[i], Protocol.ONE, Prefix(st["prefix"]), st["degree"], insts))
        for i, pb in zip(live, prove_many(jobs, device=dev)):
            st = sessions[i]["stages"][k]
            assert pb.gamma == tuple(num(x) for x in st["gamma"])
            assert pb.proof.rounds == [fp2s(m) for m in st["rounds"]], (sessions[i]["name"], st["prefix"])
            assert pb.point == fp2s(st["challenges"])
            assert pb.proof.final_evals == fp2s(st["final_evals"])
            assert ts[i].state.hex() == st["state"] and ts[i].counter == st["counter"]
            count += 1
    assert count == 62


def _spec_jobs(rng_seed):
    """Uneven jobs: several instances with front padding, prime-field, extension and public
    tables, degrees 1..7, instances on 0 variables."""
    rs = np.random.default_rng(rng_seed)
    jobs = []
    for b in range(10):
        degree = int(rs.integers(1, 8))
        specs = []
        for i in range(int(rs.integers(1, 4))):
            vars_ = int(rs.integers(0, 12))
            tables = []
            for k in range(int(rs.integers(1, degree + 1))):
                is_ext = bool(rs.integers(0, 2))
                vals = O.splitmix(1000 * b + 10 * i + k, (2 if is_ext else 1) << vars_)
                tables.append((vals, is_ext, bool(rs.integers(0, 4) == 0)))
            specs.append(tables)
        jobs.append((f"stage/{b}", degree, specs))
    return jobs


def _insts(specs):
    from tessera_gb300.sumcheck import Instance, Table

    out = []
    for spec in specs:
        tabs = []
        for v, e, p in spec:
            t = Table.ext(v) if e else Table.base(v)
            tabs.append(t.public() if p else t)
        out.append(Instance(tabs))
    return out


def test_prove_many_uneven_vs_oracle(dev):
    from tessera_gb300.hash import Transcript
    from tessera_gb300.sumcheck import Protocol, prove_many

    jobs = _spec_jobs(7)
    ts = [Transcript(ctx(b.to_bytes(16, "little"))) for b in range(len(jobs))]
    res = prove_many([(ts[b], Protocol.ONE, pre, deg, _insts(specs)) for b, (pre, deg, specs) in enumerate(jobs)],
                     device=dev)
    for b, ((pre, deg, specs), pb) in enumerate(zip(jobs, res)):
        ot = O.OracleTranscript(ctx(b.to_bytes(16, "little")).tce())
        g, rounds, chal, evals = O.prove_batch(ot, pre, deg, specs)
        assert pb.gamma == g and pb.proof.rounds == rounds and pb.point == chal and pb.proof.final_evals == evals, b
        assert ts[b].state == ot.state and ts[b].counter == ot.counter


@pytest.mark.parametrize("njobs,lo,hi", [(2, 12, 15), (7, 0, 12), (8, 11, 14), (9, 0, 12)])
def test_prove_many_job_counts_vs_oracle(dev, njobs, lo, hi):
    """Up to eight jobs keep their transcripts in every block of the persistent rounds (one meeting
    a round; with fewer than eight a spare warp fetches the next segment); nine or more take the
    owner-warp path with two meetings. Jobs of 2^lo..2^hi entries, several instances each, so that
    the larger ones have multi-block persistent rounds."""
    from tessera_gb300.hash import Transcript
    from tessera_gb300.sumcheck import Protocol, prove_many

    rs = np.random.default_rng(100 + njobs)
    jobs = []
    for b in range(njobs):
        degree = int(rs.integers(1, 5))
        specs = []
        for i in range(int(rs.integers(1, 3))):
            vars_ = int(rs.integers(lo, hi + 1))
            specs.append([(O.splitmix(5000 * b + 10 * i + k, (2 if k == 1 else 1) << vars_), k == 1, False)
                          for k in range(degree)])
        jobs.append((f"stage/{b}", degree, specs))
    ts = [Transcript(ctx(b.to_bytes(16, "little"))) for b in range(njobs)]
    res = prove_many([(ts[b], Protocol.ONE, pre, deg, _insts(specs)) for b, (pre, deg, specs) in enumerate(jobs)],
                     device=dev)
    for b, ((pre, deg, specs), pb) in enumerate(zip(jobs, res)):
        ot = O.OracleTranscript(ctx(b.to_bytes(16, "little")).tce())
        g, rounds, chal, evals = O.prove_batch(ot, pre, deg, specs)
        assert pb.gamma == g and pb.proof.rounds == rounds and pb.point == chal and pb.proof.final_evals == evals, b
        assert ts[b].state == ot.state and ts[b].counter == ot.counter


def _batched_jobs(max_vars, count=64):
    from tessera_gb300.workloads import batched, splitmix_words

    _, shapes = batched(0x00650003, commitments=0, sumchecks=count, max_vars=max_vars)
    return [(s, [splitmix_words(s.seed + i, 1 << s.vars) for i in range(s.degree)]) for s in shapes]


@pytest.mark.parametrize("max_vars", [14, 22])
def test_prove_many_batched_workload_vs_plain(dev, max_vars):
    """The batched workload's 64 sumchecks (variables 10..22, degree 2 or 3, one transcript each)
    proved together equal the plain path, one prove_batch per job; at up to 2^14 entries the
    first eight also match the oracle."""
    from tessera_gb300.hash import Transcript
    from tessera_gb300.sumcheck import Instance, Protocol, Table, prove_batch, prove_many

    jobs = _batched_jobs(max_vars)
    tb = [Transcript(ctx(s.session_id)) for s, _ in jobs]
    together = prove_many([(tb[i], Protocol.ONE, "stage/0", s.degree, [Instance([Table.base(x) for x in tabs])])
                           for i, (s, tabs) in enumerate(jobs)], device=dev)
    for i, (s, tabs) in enumerate(jobs):
        t = Transcript(ctx(s.session_id))
        alone = prove_batch(t, Protocol.ONE, "stage/0", s.degree, [Instance([Table.base(x) for x in tabs])], device=dev)
        assert together[i] == alone, i
        assert tb[i].state == t.state and tb[i].counter == t.counter
        if max_vars <= 14 and i < 8:
            ot = O.OracleTranscript(ctx(s.session_id).tce())
            g, rounds, chal, evals = O.prove_batch(ot, "stage/0", s.degree, [[(x, False, False) for x in tabs]])
            assert (alone.gamma, alone.proof.rounds, alone.point, alone.proof.final_evals) == (g, rounds, chal, evals)


def test_prove_many_many_small_jobs_vs_oracle(dev):
    """200 small jobs (4..9 variables, degree 2 or 3) in one prove_many: more jobs than the
    persistent rounds' warps, so each job's transcript state goes through device memory between
    rounds; every job equals the CPU oracle's proof on its own transcript."""
    from tessera_gb300.hash import Transcript
    from tessera_gb300.sumcheck import Instance, Protocol, Table, prove_many
    from tessera_gb300.workloads import splitmix_words

    rs = np.random.default_rng(11)
    specs = []
    for b in range(200):
        vars_, degree = int(rs.integers(4, 10)), int(rs.integers(2, 4))
        specs.append((vars_, degree, [splitmix_words(0x9100 + 7 * b + i, 1 << vars_) for i in range(degree)]))
    ts = [Transcript(ctx(b.to_bytes(16, "little"))) for b in range(len(specs))]
    res = prove_many([(ts[b], Protocol.ONE, "stage/0", deg, [Instance([Table.base(x) for x in tabs])])
                      for b, (_, deg, tabs) in enumerate(specs)], device=dev)
    for b, ((_, deg, tabs), pb) in enumerate(zip(specs, res)):
        ot = O.OracleTranscript(ctx(b.to_bytes(16, "little")).tce())
        g, rounds, chal, evals = O.prove_batch(ot, "stage/0", deg, [[(x, False, False) for x in tabs]])
        assert (pb.gamma, pb.proof.rounds, pb.point, pb.proof.final_evals) == (g, rounds, chal, evals), b
        assert ts[b].state == ot.state and ts[b].counter == ot.counter


def test_prove_many_device_tables(dev):
    """Tables already in device memory (torch tensors) go through without copies."""
    import torch

    from tessera_gb300.hash import Transcript
    from tessera_gb300.sumcheck import Instance, Protocol, Table, prove_batch, prove_many

    jobs = _batched_jobs(12, count=6)
    tb = [Transcript(ctx(s.session_id)) for s, _ in jobs]
    dtabs = [[torch.from_numpy(x.view(np.int64)).to(f"cuda:{dev.ordinal}") for x in tabs] for _, tabs in jobs]
    together = prove_many([(tb[i], Protocol.ONE, "stage/0", s.degree, [Instance([Table.base(x) for x in dtabs[i]])])
                           for i, (s, _) in enumerate(jobs)], device=dev)
    for i, (s, tabs) in enumerate(jobs):
        t = Transcript(ctx(s.session_id))
        assert together[i] == prove_batch(t, Protocol.ONE, "stage/0", s.degree, [Instance([Table.base(x) for x in tabs])],
                                          device=dev)


def test_prove_many_refusal_leaves_transcripts(dev):
    """A malformed job (degree 0) refuses the whole call before any transcript moves."""
    from tessera_gb300 import _native as N
    from tessera_gb300.hash import Transcript
    from tessera_gb300.sumcheck import Instance, Protocol, Table, prove_many

    jobs = _batched_jobs(10, count=3)
    ts = [Transcript(ctx(s.session_id)) for s, _ in jobs]
    before = [(t.state, t.counter) for t in ts]
    call = [(ts[i], Protocol.ONE, "stage/0", s.degree, [Instance([Table.base(x) for x in tabs])])
            for i, (s, tabs) in enumerate(jobs)]
    call[2] = (ts[2], Protocol.ONE, "stage/0", 0, call[2][4])
    with pytest.raises(N.TesseraError):
        prove_many(call, device=dev)
    assert [(t.state, t.counter) for t in ts] == before


# ---- commitments --------------------------------------------------------------------------------

def _commit_inputs(dev, max_log_k, max_polys, count=64):
    import torch

    from tessera_gb300.pcs import CommitmentParams
    from tessera_gb300.workloads import batched, splitmix_words

    shapes, _ = batched(0x00650003, commitments=count, sumchecks=0, max_log_k=max_log_k, max_polys=max_polys)
    params = [CommitmentParams(s.log_k, s.log_inv_rate, 0, 32, s.commitment_id) for s in shapes]
    rows = [torch.from_numpy(splitmix_words(s.seed, s.polys << s.log_k).view(np.int64)).to(f"cuda:{dev.ordinal}")
            for s in shapes]
    return params, rows


def _plain(dev, p, rows):
    """The plain path: one tg_commit_unmasked_dev call."""
    import ctypes

    import torch

    from tessera_gb300 import _native as N

    k, n = 1 << p.log2_k, 1 << (p.log2_k + p.log2_inv_rate)
    npolys = rows.numel() // k
    cw = torch.empty(max(npolys * n, 1), dtype=torch.int64, device=rows.device)
    nodes = torch.empty((2 * n - 1) * 32, dtype=torch.uint8, device=rows.device)
    root = ctypes.create_string_buffer(32)
    cid = (ctypes.c_uint8 * 32)(*p.commitment_id)
    torch.cuda.current_stream().synchronize()
    N.call("tg_commit_unmasked_dev", dev.handle, p.log2_k, p.log2_inv_rate, p.row_block, cid,
           ctypes.c_void_p(rows.data_ptr()), npolys, ctypes.c_void_p(cw.data_ptr()), ctypes.c_void_p(nodes.data_ptr()),
           root, None)
    return root.raw, nodes, cw


@pytest.mark.parametrize("workers", [0, 1, 3, 8])
def test_commit_many_vs_plain(dev, workers):
    """64 commitments of the batched workload's uneven shapes (k up to 2^14, up to 32 rows) on
    several streams equal the plain path, node for node and codeword for codeword."""
    import torch

    from tessera_gb300.pcs import commit_many

    params, rows = _commit_inputs(dev, 14, 32)
    res = commit_many(params, rows, device=dev, workers=workers)
    for p, r, c in zip(params, rows, res):
        root, nodes, cw = _plain(dev, p, r)
        assert c.root == root
        assert torch.equal(c.nodes, nodes) and torch.equal(c.codewords, cw)


def test_commit_many_vs_oracle(dev):
    from tessera_gb300.pcs import commit_many

    params, rows = _commit_inputs(dev, 13, 8, count=12)
    res = commit_many(params, rows, device=dev)
    for p, r, c in zip(params, rows, res):
        host = r.cpu().numpy().view(np.uint64)
        _, leaves, root = O.commit_unmasked(host, p.log2_k, p.log2_inv_rate, 32, p.commitment_id,
                                            threads=O.threads_available(), keep_codewords=False)
        assert c.root == root and b"".join(c.leaves()) == leaves.tobytes()


def test_commit_plan_replays(dev):
    """A captured plan (worker count autotuned) equals the plain path, and a second launch after
    the rows were overwritten in place commits the new contents."""
    import torch

    from tessera_gb300.pcs import CommitPlan
    from tessera_gb300.workloads import splitmix_words

    params, rows = _commit_inputs(dev, 15, 128, count=24)
    plan = CommitPlan(params, rows, device=dev)
    try:
        info = plan.info()
        assert info["workers"] in (1, 2, 4, 8) and info["kernels_per_launch"] > 0
        assert set(info["tuned_ms"]) == {1, 2, 4, 8}
        for rnd in range(2):
            if rnd:
                for i, r in enumerate(rows):
                    r.copy_(torch.from_numpy(splitmix_words(0xABC + i, r.numel()).view(np.int64)).to(r.device))
            roots = plan.launch()
            for p, r, c, root in zip(params, rows, plan.commitments, roots):
                proot, nodes, cw = _plain(dev, p, r)
                assert root == proot and torch.equal(c.nodes, nodes) and torch.equal(c.codewords, cw)
    finally:
        plan.close()


def test_commit_plan_tuning_cache(dev, tmp_path, monkeypatch):
    """Encoder configurations read from the tuning cache — splits of the row transform other than
    the default (columns of 2,048 in passes A/C or M1/M2 among them) and groups of one to three
    rows — commit exactly what the plain path commits; a plan over shapes missing from the cache
    times their candidates and appends one line per shape."""
    import torch

    from tessera_gb300.pcs import CommitmentParams, CommitPlan
    from tessera_gb300.workloads import splitmix_words

    sm = torch.cuda.get_device_properties(dev.ordinal).multi_processor_count
    # (log k, log inverse rate, rows, log K1, rows per group)
    forced = [(13, 1, 4, 7, 2), (16, 1, 8, 7, 3), (19, 2, 4, 11, 1), (20, 1, 2, 9, 1), (21, 1, 2, 10, 1)]
    cache = tmp_path / "tune.txt"
    cache.write_text("".join(f"encode {sm} {lk} {lr} {np_} {c} {g} 1.0 1.0\n" for lk, lr, np_, c, g in forced)
                     + "encode 1 13 1 4 6 1 1.0 1.0\nnot a line\n")
    monkeypatch.setenv("TESSERA_GB300_TUNE_CACHE", str(cache))
    params = [CommitmentParams(lk, lr, 0, 32, bytes([lk]) * 32) for lk, lr, _, _, _ in forced]
    rows = [torch.from_numpy(splitmix_words(0x7700 + i, np_ << lk).view(np.int64)).to(f"cuda:{dev.ordinal}")
            for i, (lk, _, np_, _, _) in enumerate(forced)]
    plan = CommitPlan(params, rows, device=dev, workers=2)
    try:
        shapes = {(s["log_k"], s["log_inv_rate"], s["rows"]): s for s in plan.info()["encoder_shapes"]}
        for lk, lr, np_, c, g in forced:
            s = shapes[(lk, lr, np_)]
            assert s["from_cache"] and s["split_log"] == c and s["group"] == g
        for p, r, c, root in zip(params, rows, plan.commitments, plan.launch()):
            proot, nodes, cw = _plain(dev, p, r)
            assert root == proot and torch.equal(c.nodes, nodes) and torch.equal(c.codewords, cw)
    finally:
        plan.close()
    before = cache.read_text().count("\n")
    extra = [CommitmentParams(15, 2, 0, 32, bytes(32))]
    xrows = [torch.from_numpy(splitmix_words(0x7800, 16 << 15).view(np.int64)).to(f"cuda:{dev.ordinal}")]
    plan = CommitPlan(extra, xrows, device=dev, workers=1)
    try:
        (s,) = plan.info()["encoder_shapes"]
        assert not s["from_cache"] and s["candidates"] >= 2 and s["ms_tuned"] <= s["ms_default"]
        assert plan.launch()[0] == _plain(dev, extra[0], xrows[0])[0]
    finally:
        plan.close()
    lines = cache.read_text().splitlines()
    assert len(lines) == before + 1 and lines[-1].startswith(f"encode {sm} 15 2 16 ")


def test_commit_many_large_shapes(dev):
    """The batched workload with k up to 2^18 and up to 128 rows per commitment: batched equals
    plain on every root."""
    from tessera_gb300.pcs import commit_many

    params, rows = _commit_inputs(dev, 18, 128, count=32)
    res = commit_many(params, rows, device=dev)
    for p, r, c in zip(params, rows, res):
        assert c.root == _plain(dev, p, r)[0]


def test_commit_many_refusals(dev):
    import torch

    from tessera_gb300 import _native as N
    from tessera_gb300.pcs import CommitmentParams, commit_many

    rows = torch.zeros(4 << 10, dtype=torch.int64, device=f"cuda:{dev.ordinal}")
    for bad in (CommitmentParams(10, 0, 0, 32, bytes(32)), CommitmentParams(10, 5, 0, 32, bytes(32)),
                CommitmentParams(10, 1, 0, 0, bytes(32)), CommitmentParams(10, 1, 0, 125, bytes(32))):
        with pytest.raises(N.TesseraError):
            commit_many([CommitmentParams(10, 1, 0, 32, bytes(32)), bad], [rows, rows], device=dev)


def test_fill_splitmix_matches_host(dev):
    """The device generator of synthetic inputs equals the host SplitMix64 words."""
    import torch

    from tessera_gb300.workloads import fill_device, splitmix_words

    for seed, n in ((0, 1), (0x00650003, 12345), (2**64 - 1, 1 << 20)):
        t = fill_device(torch.empty(n, dtype=torch.int64, device=f"cuda:{dev.ordinal}"), seed, dev)
        assert (t.cpu().numpy().view(np.uint64) == splitmix_words(seed, n)).all()
