"""GPU parity of the batched sumcheck, the tree-level offload and proof-of-work grinding against
the reference's golden vectors and the CPU oracle: every round message, challenge, final
evaluation and transcript state, bit for bit."""
import numpy as np
import pytest

from golden_data import context_tce, fp2s, load, num, stage_tables
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dev():
    from tessera_gb300.device import default_device

    return default_device()


def test_sumcheck_golden_stages(dev):
    """All 62 stages of the reference's sumcheck sessions: degrees 1 to 7, front padding,
    batches of equal sizes, n_max = 0, several stages on one transcript."""
    from tessera_gb300.hash import Transcript
    from tessera_gb300.sumcheck import Instance, Prefix, Protocol, Table, prove_batch

    v = load("sumcheck")
    seed = num(v["seed"])
    count = 0
    for session in v["sessions"]:
        t = Transcript(context_tce(session["context"]))
        for st in session["stages"]:
            tables = stage_tables(seed, st)
            insts = [Instance([Table.ext(tb) for tb in inst]) for inst in tables]
            pb = prove_batch(t, Protocol.ONE, Prefix(st["prefix"]), st["degree"], insts, device=dev)
            assert pb.gamma == tuple(num(x) for x in st["gamma"])
            assert pb.proof.rounds == [fp2s(m) for m in st["rounds"]], (session["name"], st["prefix"])
            assert pb.point == fp2s(st["challenges"])
            assert pb.proof.final_evals == fp2s(st["final_evals"])
            assert t.state.hex() == st["state"] and t.counter == st["counter"]
            count += 1
    assert count == 62


def bench_context():
    from tessera_gb300.hash import Mode, SessionContext

    return SessionContext("tessera-protocol/1", Mode.NON_INTERACTIVE, "test-small/1", bytes([0x65]) * 32, bytes([0x65]) * 16)


def run_both(dev, prefix, degree, specs):
    """specs: per instance, a list of (values, is_ext, is_public)."""
    from tessera_gb300.hash import Transcript
    from tessera_gb300.sumcheck import Instance, Protocol, Table, prove_batch

    ctx = bench_context()
    t = Transcript(ctx)
    insts = [Instance([(Table.ext(v) if e else Table.base(v)).public() if p else (Table.ext(v) if e else Table.base(v))
                       for v, e, p in spec]) for spec in specs]
    pb = prove_batch(t, Protocol.ONE, prefix, degree, insts, device=dev)
    ot = O.OracleTranscript(ctx.tce())
    g, rounds, chal, evals = O.prove_batch(ot, prefix, degree, specs)
    assert pb.gamma == g
    assert pb.proof.rounds == rounds
    assert pb.point == chal
    assert pb.proof.final_evals == evals
    assert t.state == ot.state and t.counter == ot.counter
    return pb


def test_sumcheck_fg_2p14(dev):
    """Σ f·g over two prime-field tables of 2^14 entries, degree 2: 14 rounds."""
    f, g = O.splitmix(1, 1 << 14), O.splitmix(2, 1 << 14)
    run_both(dev, "stage/0", 2, [[(f, False, False), (g, False, False)]])


def test_sumcheck_fgh_2p22(dev):
    """Σ f·g·h over three prime-field tables of 2^22 entries, degree 3: 22 rounds."""
    f, g, h = (O.splitmix(s, 1 << 22) for s in (3, 4, 5))
    run_both(dev, "stage/0", 3, [[(f, False, False), (g, False, False), (h, False, False)]])


@pytest.mark.parametrize("degree", [2, 3])
@pytest.mark.parametrize("log_len", [3, 4, 6, 9, 12, 17])
def test_sumcheck_one_instance_small_rounds(dev, degree, log_len):
    """One instance of `degree` tables at that degree: every round of at most 2^16 pairs runs in the
    persistent launch, and from round 2 the one-block rounds of at most 32 pairs take their sums from
    the look-ahead (round t+1's sums as a polynomial in r_t, written while r_t is drawn). Prime-field
    and Fp2 tables, one of them public."""
    n = 1 << log_len
    specs = [[(O.splitmix(40 + k, (2 if k == 1 else 1) * n), k == 1, k == degree - 1) for k in range(degree)]]
    run_both(dev, "stage/2", degree, specs)


def test_sumcheck_mixed_public_padded(dev):
    """Prime-field and Fp2 tables in one product, a public factor, front padding, a constant."""
    specs = [
        [(O.splitmix(10, 1 << 9), False, False), (O.splitmix(11, 2 << 9), True, False), (O.splitmix(12, 1 << 9), False, True)],
        [(O.splitmix(13, 1 << 4), False, False)],
        [(O.splitmix(14, 2), True, False), (O.splitmix(15, 1), False, False)],
        [(O.splitmix(16, 1 << 9), False, False), (O.splitmix(17, 1 << 9), False, False)],
    ]
    run_both(dev, "stage/3", 4, specs)


@pytest.mark.parametrize("degree", [1, 5, 7])
def test_sumcheck_degrees(dev, degree):
    specs = [[(O.splitmix(20 + k, 1 << 11), False, False) for k in range(degree)]]
    run_both(dev, "stage/1", degree, specs)


def test_sumcheck_device_tables(dev):
    """Tables already in device memory give the same proof as host tables."""
    import torch

    from tessera_gb300.hash import Transcript
    from tessera_gb300.sumcheck import Instance, Protocol, Table, prove_batch

    f, g = O.splitmix(41, 1 << 16), O.splitmix(42, 1 << 16)
    t1, t2 = Transcript(bench_context()), Transcript(bench_context())
    a = prove_batch(t1, Protocol.ONE, "stage/0", 2, [Instance([Table.base(f), Table.base(g)])], device=dev)
    df = torch.from_numpy(f.view(np.int64)).cuda()
    dg = torch.from_numpy(g.view(np.int64)).cuda()
    b = prove_batch(t2, Protocol.ONE, "stage/0", 2, [Instance([Table.base(df), Table.base(dg)])], device=dev)
    assert a.proof == b.proof and t1.state == t2.state


def test_sumcheck_refusals_leave_transcript(dev):
    from tessera_gb300 import _native as N
    from tessera_gb300.hash import Transcript
    from tessera_gb300.sumcheck import Instance, Protocol, Table, prove_batch

    t = Transcript(bench_context())
    s0 = t.state
    f = O.splitmix(1, 8)
    for degree, insts in [(0, [Instance([Table.base(f)])]), (8, [Instance([Table.base(f)])]),
                          (1, [Instance([Table.base(f), Table.base(f)])]), (2, [])]:
        with pytest.raises(N.InvalidInput):
            prove_batch(t, Protocol.ONE, "stage/0", degree, insts, device=dev)
    with pytest.raises(N.InvalidInput):
        prove_batch(t, Protocol.ONE, "stage/0", 2, [Instance([Table.base(f), Table.base(f[:4])])], device=dev)
    assert t.state == s0 and t.counter == 0


# ---- tree-level offload -------------------------------------------------------------------------

def fp2_table(seed, n):
    return O.splitmix(seed, 2 * n)


@pytest.mark.parametrize("shape,log_len,low_bits", [("fraction", 14, 5), ("product", 15, 7), ("fraction", 16, 0),
                                                    ("product", 14, 13)])
def test_level_rounds_match_oracle(dev, shape, log_len, low_bits):
    from tessera_gb300.offload import GpuLevels, LevelShape

    n = 1 << log_len
    nt = 4 if shape == "fraction" else 2
    tables = [fp2_table(100 + k, n) for k in range(nt)]
    lam = (int(O.splitmix(7, 1)[0]), int(O.splitmix(8, 1)[0]))
    ls = LevelShape.fraction(lam) if shape == "fraction" else LevelShape.product()
    lvl = GpuLevels(dev).load(ls, tables)
    assert lvl is not None
    cur = [t.copy() for t in tables]
    length = n
    rnd = 0
    while length >= 2:
        npairs = length // 2
        lb = min(low_bits, max(0, npairs.bit_length() - 1))
        low = fp2_table(200 + rnd, 1 << lb)
        high = fp2_table(300 + rnd, max(1, npairs >> lb))
        got = lvl.sums(low, high, lb)
        want = O.level_sums(shape, lam, cur, low, high, lb)
        assert got == want, (rnd, length)
        r = (int(O.splitmix(400 + rnd, 1)[0]), int(O.splitmix(500 + rnd, 1)[0]))
        lvl.bind(r)
        cur = O.level_bind(cur, r)
        length //= 2
        rnd += 1
        if rnd == 3 and length >= 4:  # two binds in a row, no sums between
            r2 = (5, 6)
            lvl.bind(r2)
            cur = O.level_bind(cur, r2)
            length //= 2
    assert lvl.firsts() == [(int(t[0]), int(t[1])) for t in cur]
    lvl.close()


def test_level_declines(dev):
    from tessera_gb300.offload import GpuLevels, LevelShape

    small = [fp2_table(k, 1 << 10) for k in range(2)]
    assert GpuLevels(dev).load(LevelShape.product(), small) is None  # below 2^14 entries
    assert GpuLevels(dev).load(LevelShape.product(), [fp2_table(1, 1 << 14)] * 3) is None  # wrong table count


# ---- proof of work --------------------------------------------------------------------------------

def test_grind_golden(dev):
    from tessera_gb300.hash import Transcript

    seen = 0
    for c in load("transcript")["cases"]:
        t = Transcript(bytes.fromhex(c["context_tce"]))
        for s in c["steps"]:
            op = s["op"]
            if op == "absorb":
                t.absorb(s["label"], bytes.fromhex(s["tce"]))
            elif op == "squeeze":
                t.squeeze(s["label"])
            elif op == "challenge_fp2":
                t.challenge_fp2(s["label"])
            elif op == "challenge_fp":
                t.challenge_fp(s["label"])
            elif op == "challenge_indices":
                t.challenge_indices(s["label"], s["log_n"], s["count"])
            elif op == "grind":
                assert t.grind(s["label"], s["bits"], device=dev) == num(s["nonce"])
                seen += 1
            elif op == "check_grind":
                t.check_grind(s["label"], s["bits"], num(s["nonce"]))
            assert t.state.hex() == s["state"]
    assert seen >= 4


def test_grind_matches_oracle_20_bits(dev):
    from tessera_gb300.hash import Transcript

    t = Transcript(bench_context())
    ot = O.OracleTranscript(bench_context().tce())
    assert t.grind("query-pow", 16, device=dev) == ot.grind("query-pow", 16)
    assert t.state == ot.state


def test_persistent_rounds_meetings_are_bounded(dev):
    """The persistent rounds' blocks meet between rounds with bounded waits: 64 blocks meet 200
    times; with one block gone before the first meeting, the others give up after their polls, the
    meeting point records it, and the call returns (no block waits for good)."""
    import ctypes
    import time

    from tessera_gb300 import _native as N

    met, gave = ctypes.c_int(), ctypes.c_int()
    N.call("tg_check_grid_meet", dev.handle, 64, 200, -1, 1 << 22, ctypes.byref(met), ctypes.byref(gave))
    assert (met.value, gave.value) == (64, 0)
    t0 = time.perf_counter()
    N.call("tg_check_grid_meet", dev.handle, 64, 200, 5, 1 << 14, ctypes.byref(met), ctypes.byref(gave))
    assert (met.value, gave.value) == (0, 1)
    assert time.perf_counter() - t0 < 10
    with pytest.raises(N.TesseraError):
        N.call("tg_check_grid_meet", dev.handle, 64, 1, 64, 1 << 14, ctypes.byref(met), ctypes.byref(gave))
