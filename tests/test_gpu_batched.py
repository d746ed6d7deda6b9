"""The batched pattern on the GPU: many independent sumchecks proved together (one fused launch
per round for all of them) give, byte for byte, what one-at-a-time proofs give — checked against
the reference's golden sessions, the CPU oracle and the plain per-job path, on the batched
workload's uneven shapes."""
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
