"""GPU parity of the commitment path against the CPU oracle and the reference's golden vectors:
Reed–Solomon encoding (every shape class, masks, rates 1/2 to 1/16), column chains, Merkle
trees, the resident unmasked commitment (the 32 x 2^14 and 256 x 2^20 workloads), the advice
BlockSink with segment merging, the MatrixSink, and the opening's ColumnSink (queried columns and
combined rows). Bit-exact throughout."""
import os

import numpy as np
import pytest

from golden_data import load, num
from oracle import oracle as O

pytestmark = pytest.mark.gpu

THREADS = O.threads_available()


@pytest.fixture(scope="module")
def dev():
    from tessera_gb300.device import default_device

    return default_device()


def rand_fp(seed, n):
    return O.splitmix(seed, n)


# ---- encoding ---------------------------------------------------------------------------------

def test_encoding_golden(dev):
    from tessera_gb300.pcs import RowEncoder

    for c in load("encoding")["encoding"]:
        k = c["k"]
        log_r = (len(c["codeword"]) // k).bit_length() - 1
        enc = RowEncoder(k, log_r, c["mask_coeffs"], device=dev)
        cw = enc.encode_rows([num(x) for x in c["row"]], [num(x) for x in c["mask"]])
        assert [int(x) for x in cw[0]] == [num(x) for x in c["codeword"]]


def test_coset_values_golden(dev):
    """A row of f(ω_n^i) encoded at rate 1/2: its even symbols are f(7 ω_n^q)."""
    from tessera_gb300.pcs import RowEncoder

    for c in load("encoding")["ntt"]:
        n = c["n"]
        cw = RowEncoder(n, 1, device=dev).encode_rows([num(x) for x in c["values"]])[0]
        assert [int(x) for x in cw[0::2]] == [num(x) for x in c["coset_values"]]


@pytest.mark.parametrize("log_k", [0, 1, 2, 3, 5, 8, 10, 11, 12, 13, 14, 15, 16, 17])
@pytest.mark.parametrize("log_r", [1, 2, 3, 4])
def test_encode_matches_oracle(dev, log_k, log_r):
    from tessera_gb300.pcs import RowEncoder

    if log_k + log_r > 20:
        pytest.skip("covered by the large shapes")
    k = 1 << log_k
    nrows = 3
    rows = rand_fp(1000 + 17 * log_k + log_r, nrows * k)
    for P in sorted({0, 1, k // 2, k}):
        masks = rand_fp(77 + P, nrows * P) if P else None
        got = RowEncoder(k, log_r, P, device=dev).encode_rows(rows, masks)
        want = O.encode_rows(rows, log_k, log_r, masks=masks, mask_coeffs=P, threads=THREADS)
        assert np.array_equal(got, want), (log_k, log_r, P)


@pytest.mark.parametrize("log_k,log_r,nrows,P", [(20, 1, 2, 0), (20, 1, 1, 200), (21, 1, 1, 0), (22, 1, 1, 200),
                                                 (21, 2, 2, 7), (22, 3, 1, 0), (22, 1, 3, 1),
                                                 (18, 2, 2, 0), (23, 1, 1, 0), (24, 1, 1, 5)])
def test_encode_large_matches_oracle(dev, log_k, log_r, nrows, P):
    from tessera_gb300.pcs import RowEncoder

    k = 1 << log_k
    rows = rand_fp(5 + log_k, nrows * k)
    masks = rand_fp(9, nrows * P) if P else None
    got = RowEncoder(k, log_r, P, device=dev).encode_rows(rows, masks)
    want = O.encode_rows(rows, log_k, log_r, masks=masks, mask_coeffs=P, threads=THREADS)
    assert np.array_equal(got, want)


def test_encode_edge_values(dev):
    """Rows of 0, 1 and p − 1 everywhere, and alternating extremes."""
    from tessera_gb300.pcs import RowEncoder

    P_ = O.P
    for log_k in (4, 12, 14):
        k = 1 << log_k
        rows = np.concatenate([np.zeros(k, np.uint64), np.ones(k, np.uint64), np.full(k, P_ - 1, np.uint64),
                               np.tile(np.array([0, P_ - 1], np.uint64), k // 2)])
        got = RowEncoder(k, 1, device=dev).encode_rows(rows)
        assert np.array_equal(got, O.encode_rows(rows, log_k, 1))


def test_encode_refuses_bad_shapes(dev):
    from tessera_gb300 import _native as N
    from tessera_gb300.pcs import RowEncoder

    with pytest.raises(ValueError):
        RowEncoder(3, 1, device=dev)
    with pytest.raises(ValueError):
        RowEncoder(8, 0, device=dev)
    with pytest.raises(ValueError):
        RowEncoder(8, 1, 9, device=dev)
    with pytest.raises(ValueError):
        RowEncoder(8, 1, device=dev).encode_rows(np.zeros(12, np.uint64))


# ---- hashing ----------------------------------------------------------------------------------

def test_column_chains_golden(dev):
    from tessera_gb300.hash import ColumnChains

    for c in load("hash")["columns"]:
        rows = np.array([[num(x) for x in r] for r in c["rows"]], dtype=np.uint64)
        ch = ColumnChains(bytes.fromhex(c["commitment_id"]), c["columns"], c["block"], device=dev)
        for b in range(0, len(rows), c["block"]):
            ch.absorb_block(rows[b:b + c["block"]])
        assert [x.hex() for x in ch.finish()] == c["leaves"]


@pytest.mark.parametrize("block,m,ncols", [(1, 3, 5), (3, 7, 64), (32, 32, 4096), (32, 77, 1000), (124, 124, 300),
                                           (124, 250, 513), (5, 1, 2)])
def test_column_chains_match_oracle(dev, block, m, ncols):
    from tessera_gb300.hash import ColumnChains

    cid = bytes(range(32))
    rows = rand_fp(block * 1000 + m, m * ncols).reshape(m, ncols)
    ch = ColumnChains(cid, ncols, block, device=dev)
    for b in range(0, m, block):
        ch.absorb_block(rows[b:b + block])
    want = O.column_chains(cid, rows, ncols, block, threads=THREADS)
    assert b"".join(ch.finish()) == want.tobytes()


def test_column_chains_refuse_blocks(dev):
    from tessera_gb300 import _native as N
    from tessera_gb300.hash import ColumnChains

    ch = ColumnChains(bytes(32), 4, 3, device=dev)
    with pytest.raises(ValueError):
        ch.absorb_block(np.zeros(16, np.uint64))  # 4 rows > B
    ch.absorb_block(np.zeros(8, np.uint64))  # short block: the last
    with pytest.raises(N.TesseraError):
        ch.absorb_block(np.zeros(4, np.uint64))


def test_merkle_golden(dev):
    from tessera_gb300.hash import MerkleTree

    for m in load("hash")["merkle"]:
        t = MerkleTree([bytes.fromhex(x) for x in m["leaves"]], device=dev)
        assert t.root().hex() == m["root"]


@pytest.mark.parametrize("n", [1, 2, 4, 512, 1024, 1 << 17])
def test_merkle_matches_oracle(dev, n):
    from tessera_gb300.hash import MerkleTree

    leaves = np.frombuffer(rand_fp(n, 4 * n).tobytes(), dtype=np.uint8).reshape(n, 32)
    t = MerkleTree(leaves, device=dev)
    assert np.array_equal(t.nodes(), O.merkle_tree(leaves, threads=THREADS))


# ---- commitments ------------------------------------------------------------------------------

def test_commit_unmasked_32x2p14(dev):
    """The 32-polynomial, k = 2^14, rate 1/4 workload: codeword columns chained in one block of
    B = 32 rows, leaves and root."""
    from tessera_gb300.pcs import CommitmentParams, ReferenceCommitment

    cid = bytes([0x65]) * 32
    rows = rand_fp(0x00650001, 32 << 14)
    c = ReferenceCommitment.commit_unmasked(CommitmentParams(14, 2, 0, 32, cid), rows, device=dev)
    _, leaves, root = O.commit_unmasked(rows, 14, 2, 32, cid, threads=THREADS, keep_codewords=False)
    assert c.root() == root
    assert b"".join(c.leaves()) == leaves.tobytes()


@pytest.mark.parametrize("npolys,log_k,log_r,B", [(0, 4, 1, 4), (1, 0, 1, 32), (5, 6, 3, 2), (37, 10, 1, 4),
                                                  (64, 12, 2, 32), (130, 8, 1, 124)])
def test_commit_unmasked_shapes(dev, npolys, log_k, log_r, B):
    from tessera_gb300.pcs import CommitmentParams, ReferenceCommitment

    cid = bytes(range(1, 33))
    rows = rand_fp(npolys + log_k, npolys << log_k)
    c = ReferenceCommitment.commit_unmasked(CommitmentParams(log_k, log_r, 0, B, cid), rows, device=dev)
    _, leaves, root = O.commit_unmasked(rows, log_k, log_r, B, cid, threads=THREADS)
    assert c.root() == root and b"".join(c.leaves()) == leaves.tobytes()


@pytest.mark.parametrize("npolys,B,group_rows", [(37, 2, 5), (37, 3, 5), (20, 7, 5), (16, 4, 8), (9, 32, 2),
                                                 (40, 32, 40), (3, 1, 3)])
def test_commit_unmasked_pipelined_chunks(npolys, B, group_rows):
    """The host-buffer commitment copies rows in chunks of whole row blocks while the previous
    chunk encodes, and the first chunk in pieces of 1/8, 1/8, 1/4 and the rest: a small encoder
    group forces many chunks (and a short last one); the root and leaves match the oracle."""
    from tessera_gb300.device import Device
    from tessera_gb300.pcs import CommitmentParams, ReferenceCommitment

    log_k, log_r = 12, 2
    per_row = ((1 << log_k) + (1 << (log_k + log_r))) * 8
    d = Device(0, lde_group_bytes=group_rows * per_row)
    try:
        cid = bytes(range(7, 39))
        rows = rand_fp(0x5EED + npolys * B, npolys << log_k)
        _, leaves, root = O.commit_unmasked(rows, log_k, log_r, B, cid, threads=THREADS)
        for _ in range(2):  # the staging buffers are reused by the second call
            c = ReferenceCommitment.commit_unmasked(CommitmentParams(log_k, log_r, 0, B, cid), rows, device=d)
            assert c.root() == root and b"".join(c.leaves()) == leaves.tobytes()
    finally:
        d.close()


def test_commit_unmasked_256x2p20(dev):
    """The 256-polynomial, k = 2^20, rate 1/2 workload in full: 2^21 columns chained over 8
    blocks of 32 rows, and the root over 2^21 leaves."""
    from tessera_gb300.pcs import CommitmentParams, ReferenceCommitment

    cid = bytes([0x65]) * 32
    rows = rand_fp(0x00650002, 256 << 20)
    c = ReferenceCommitment.commit_unmasked(CommitmentParams(20, 1, 0, 32, cid), rows, device=dev)
    _, leaves, root = O.commit_unmasked(rows, 20, 1, 32, cid, threads=THREADS, keep_codewords=False)
    assert c.root() == root
    assert b"".join(c.leaves()) == leaves.tobytes()


def test_streaming_golden(dev):
    """The reference's segmented, masked advice commitments through the BlockSink, block by
    block, then merge_segments."""
    from tessera_gb300.pcs import AdviceSink, CommitmentParams, merge_segments

    for c in load("streaming")["cases"]:
        log_k = c["layout"]["log2_k"]
        k, n = 1 << log_k, len(c["leaves"])
        log_r = (n // k).bit_length() - 1
        rows = [[num(x) for x in r] for r in c["rows"]]
        masks = [[num(x) for x in r] for r in c["masks"]]
        params = CommitmentParams(log_k, log_r, c["mask_coeffs"], c["row_block"], bytes.fromhex(c["commitment_id"]))
        parts, off = [], 0
        for s, expected in zip(c["segments"], c["segment_digests"]):
            sink = AdviceSink(params, device=dev)
            seg_rows, seg_masks = rows[off:off + len(s)], masks[off:off + len(s)]
            for b in range(0, len(s), c["row_block"]):
                sink.absorb(seg_rows[b:b + c["row_block"]], seg_masks[b:b + c["row_block"]])
            got = sink.finish()
            sink.close()
            assert [x.hex() for x in got] == expected, c["name"]
            parts.append(got)
            off += len(s)
        merged = merge_segments(parts, device=dev)
        assert [x.hex() for x in merged.leaves] == c["leaves"]
        assert merged.root.hex() == c["root"]


def test_advice_sink_masked_rate_half_matches_oracle(dev):
    """P = 200 masks at k = 2^12, B = 32: the production advice shape, one segment."""
    from tessera_gb300.pcs import AdviceSink, CommitmentParams

    log_k, P, B, m = 12, 200, 32, 70
    k = 1 << log_k
    rows = rand_fp(31, m * k).reshape(m, k)
    masks = rand_fp(32, m * P).reshape(m, P)
    cid = bytes(range(32))
    sink = AdviceSink(CommitmentParams(log_k, 1, P, B, cid), device=dev)
    for b in range(0, m, B):
        sink.absorb(rows[b:b + B], masks[b:b + B])
    got = b"".join(sink.finish())
    cw = O.encode_rows(rows, log_k, 1, masks=masks, mask_coeffs=P, threads=THREADS)
    want = O.column_chains(cid, cw, 2 * k, B, threads=THREADS)
    assert got == want.tobytes()


def test_advice_sink_refusals(dev):
    from tessera_gb300 import _native as N
    from tessera_gb300.pcs import AdviceSink, CommitmentParams

    sink = AdviceSink(CommitmentParams(3, 1, 2, 4, bytes(32)), device=dev)
    with pytest.raises(N.InvalidInput):
        sink.absorb(np.zeros(5 * 8, np.uint64), np.zeros(10, np.uint64))  # 5 rows > B
    sink.absorb(np.zeros(2 * 8, np.uint64), np.zeros(4, np.uint64))  # short: the last block
    with pytest.raises(N.TesseraError):
        sink.absorb(np.zeros(8, np.uint64), np.zeros(2, np.uint64))
    sink.finish()
    with pytest.raises(N.TesseraError):
        sink.finish()


@pytest.mark.parametrize("log_k,log_r,B,m", [(6, 2, 4, 10), (10, 1, 32, 33), (8, 3, 5, 5), (12, 2, 124, 124)])
def test_matrix_sink_matches_oracle(dev, log_k, log_r, B, m):
    from tessera_gb300.pcs import GpuWeights

    k = 1 << log_k
    n = k << log_r
    rows = rand_fp(log_k * 7 + m, m * k).reshape(m, k)
    queries = sorted(set(int(x) % n for x in rand_fp(3, 40)))
    cid = bytes(range(7, 39))
    sink = GpuWeights(dev).matrix(log_k, log_r, B, cid, n, queries)
    answers = []
    for b in range(0, m, B):
        answers.append(sink.absorb(rows[b:b + B]).reshape(-1, len(queries)))
    chains = b"".join(sink.finish())
    cw = O.encode_rows(rows, log_k, log_r, threads=THREADS)
    assert np.array_equal(np.concatenate(answers), cw[:, queries])
    assert chains == O.column_chains(cid, cw, n, B, threads=THREADS).tobytes()


def test_weight_encoding_declines(dev):
    from tessera_gb300.pcs import GpuWeights

    assert GpuWeights(dev).matrix(4, 1, 200, bytes(32), 32, [0]) is None  # B above one chunk
    assert GpuWeights(dev).matrix(4, 1, 4, bytes(32), 31, [0]) is None  # column count mismatch


# ---- the opening's column sink (P4/P5) ------------------------------------------------------------

def _combine_oracle(rows, coeffs, k):
    """Σ_r c[g][r]·row_r per group, with the oracle's field products (Fp2 × Fp componentwise)."""
    out = np.zeros((len(coeffs), k, 2), dtype=np.uint64)
    for g, grp in enumerate(coeffs):
        for r, (c0, c1) in enumerate(grp):
            row = rows[r * k:(r + 1) * k]
            out[g, :, 0] = O.fp_vec("add", out[g, :, 0], O.fp_vec("mul", np.full(k, c0, dtype=np.uint64), row))
            out[g, :, 1] = O.fp_vec("add", out[g, :, 1], O.fp_vec("mul", np.full(k, c1, dtype=np.uint64), row))
    return out


@pytest.mark.parametrize("log_k,log_r,P,block", [(10, 1, 0, 4), (12, 1, 5, 8), (14, 2, 1, 3), (16, 1, 64, 2)])
def test_column_sink_select_and_combine(dev, log_k, log_r, P, block):
    """The sink's queried symbols equal the oracle's encodings at those columns (including columns
    past n, which read 0), and its combined rows equal Σ_r c[g][r]·row_r over all blocks, added
    into the caller's rows."""
    from tessera_gb300.pcs import ColumnSink, RowEncoder

    k, n = 1 << log_k, 1 << (log_k + log_r)
    rng = np.random.default_rng(log_k + P)
    cols = np.concatenate([rng.integers(0, n, 37, dtype=np.uint64), np.array([n - 1, 0, n, n + 5], dtype=np.uint64)])
    enc = RowEncoder(k, log_r, P, device=dev)
    sink = ColumnSink(enc, block, cols, device=dev)
    nrows = 2 * block + 1  # two full blocks and a short one
    rows = rand_fp(log_k * 7 + P, nrows * k)
    masks = rand_fp(99 + P, nrows * P) if P else None
    groups = 3
    coeffs_all = [[tuple(int(x) for x in rand_fp(1000 * g + r, 2)) for r in range(nrows)] for g in range(groups)]
    want = O.encode_rows(rows, log_k, log_r, masks=masks, mask_coeffs=P, threads=THREADS).reshape(nrows, n)
    for r0 in range(0, nrows, block):
        r1 = min(nrows, r0 + block)
        rb = rows[r0 * k:r1 * k]
        mb = masks[r0 * P:r1 * P] if P else None
        if r0 == 0:
            got = sink.select(rb, mb)  # a block without combining contributes no sums
            coeffs_all = [[(0, 0)] * block + grp[block:] for grp in coeffs_all]
        else:
            got = sink.select_combining(rb, mb, [grp[r0:r1] for grp in coeffs_all])
        for i, c in enumerate(cols):
            expect = want[r0:r1, c] if c < n else np.zeros(r1 - r0, dtype=np.uint64)
            assert np.array_equal(got[:, i], expect)
    base = rng.integers(0, 2**32, (groups, k, 2), dtype=np.uint64)
    out = sink.combined(base.copy())
    want_sums = _combine_oracle(rows, coeffs_all, k)
    assert np.array_equal(out, O.fp_vec("add", base.reshape(-1), want_sums.reshape(-1)).reshape(base.shape))
    # collected sums are cleared: a second collection adds nothing
    again = sink.combined(base.copy())
    assert np.array_equal(again, base)
    sink.close()


def test_column_sink_refusals(dev):
    from tessera_gb300 import _native as N
    from tessera_gb300.pcs import ColumnSink, RowEncoder

    enc = RowEncoder(1 << 8, 1, 0, device=dev)
    sink = ColumnSink(enc, 2, [0, 1, 2], device=dev)
    rows = rand_fp(5, 3 << 8)
    with pytest.raises(N.TesseraError):
        sink.select(rows)  # three rows in a block of two
    sink.select_combining(rows[: 2 << 8], None, [[(1, 0), (2, 0)]])
    with pytest.raises(N.TesseraError):
        sink.select_combining(rows[: 2 << 8], None, [[(1, 0), (2, 0)], [(3, 0), (4, 0)]])  # another group count
    with pytest.raises(N.TesseraError):
        sink.combined(np.zeros((2, 1 << 8, 2), dtype=np.uint64))  # the wrong number of groups
    sink.close()
