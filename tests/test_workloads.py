"""The synthetic workloads: the SplitMix64 words equal the oracle's stream (the reference bench's
generator), and the batched workload's shapes fall in the configured ranges, deterministically."""
from oracle import oracle as O


def test_splitmix_words_match_oracle():
    from tessera_gb300.workloads import splitmix_words

    for seed in (0, 1, 0x00650002, 2**64 - 1):
        assert (splitmix_words(seed, 4096) == O.splitmix(seed, 4096)).all()


def test_batched_shapes():
    from tessera_gb300.workloads import batched

    cs, ss = batched(0x00650003)
    assert len(cs) == 64 and len(ss) == 64
    assert all(10 <= c.log_k <= 20 and c.polys in (8, 32, 128, 512) and c.log_inv_rate in (1, 2) for c in cs)
    assert all(10 <= s.vars <= 22 and s.degree in (2, 3) for s in ss)
    assert [s.session_id for s in ss] == [i.to_bytes(16, "little") for i in range(64)]
    assert batched(0x00650003) == (cs, ss)
    # caps clamp the draws without changing the sequence
    cs2, ss2 = batched(0x00650003, max_log_k=12, max_vars=14)
    assert [c.seed for c in cs2] == [c.seed for c in cs] and [s.seed for s in ss2] == [s.seed for s in ss]
    assert max(c.log_k for c in cs2) <= 12 and max(s.vars for s in ss2) <= 14
