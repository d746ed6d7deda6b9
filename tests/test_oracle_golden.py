"""Pins the CPU oracle to the reference's golden vectors (committed under tests/golden/).

Each test reproduces one conformance set of the reference (spec/vectors/...) byte for byte: the
official BLAKE3 vectors, the RFC-0004 hash domains, Merkle trees and column chains, the
transcript sessions, the RFC-0011 NTT and encodings, the streaming commitments with masks and
segments, and every sumcheck stage with its challenges, messages and final transcript state.
"""
import numpy as np
import pytest

from golden_data import blake3_input, context_tce, fp2s, load, num, stage_tables
from oracle import oracle as O

P = 0xFFFFFFFF00000001


def test_blake3_official_vectors():
    v = load("blake3")
    for c in v["cases"]:
        data = blake3_input(c["input_len"])
        assert O.blake3("hash", data, len(c["hash"]) // 2).hex() == c["hash"]
        assert O.blake3("keyed", data, len(c["keyed_hash"]) // 2, key=v["key"].encode()).hex() == c["keyed_hash"]
        assert O.blake3("derive", data, len(c["derive_key"]) // 2, key=v["context_string"]).hex() == c["derive_key"]


def test_hash_domains():
    v = load("hash")
    for d in v["domains"]:
        for n, digest in zip(v["input_lengths"], d["digests"]):
            assert O.hash_domain(d["name"], blake3_input(n)).hex() == digest, (d["name"], n)


def test_merkle_roots():
    for m in load("hash")["merkle"]:
        leaves = np.frombuffer(b"".join(bytes.fromhex(x) for x in m["leaves"]), dtype=np.uint8).reshape(-1, 32)
        assert O.merkle_root(leaves).hex() == m["root"]


def test_column_chains():
    for c in load("hash")["columns"]:
        rows = np.array([[num(x) for x in r] for r in c["rows"]], dtype=np.uint64).reshape(-1)
        chains = O.column_chains(bytes.fromhex(c["commitment_id"]), rows, c["columns"], c["block"])
        assert [bytes(x).hex() for x in chains] == c["leaves"]


def test_transcript_sessions():
    for c in load("transcript")["cases"]:
        t = O.OracleTranscript(bytes.fromhex(c["context_tce"]))
        assert t.state.hex() == c["state"]
        for s in c["steps"]:
            op = s["op"]
            if op == "absorb":
                t.absorb(s["label"], bytes.fromhex(s["tce"]))
            elif op == "squeeze":
                assert t.squeeze(s["label"]).hex() == s["out"]
            elif op == "challenge_fp2":
                assert list(t.challenge_fp2(s["label"])) == [num(x) for x in s["value"]]
            elif op == "challenge_fp":
                assert t.challenge_fp(s["label"]) == num(s["value"])
            elif op == "challenge_indices":
                assert t.challenge_indices(s["label"], s["log_n"], s["count"]) == [num(x) for x in s["value"]]
            elif op == "grind":
                assert t.grind(s["label"], s["bits"]) == num(s["nonce"])
            elif op == "check_grind":
                assert t.check_grind(s["label"], s["bits"], num(s["nonce"])) == s["valid"]
            else:
                pytest.fail(f"unknown transcript op {op}")
            assert t.state.hex() == s["state"] and t.counter == s["counter"], (c["name"], op, s["label"])


def test_ntt_vectors():
    for c in load("encoding")["ntt"]:
        coeffs = [num(x) for x in c["coefficients"]]
        assert list(O.ntt(coeffs)) == [num(x) for x in c["values"]]
        assert list(O.ntt(coeffs, coset=7)) == [num(x) for x in c["coset_values"]]
        assert list(O.ntt([num(x) for x in c["values"]], inverse=True)) == coeffs
        assert list(O.ntt([num(x) for x in c["coset_values"]], coset=7, inverse=True)) == coeffs


def test_encoding_vectors():
    for c in load("encoding")["encoding"]:
        k = c["k"]
        log_k = k.bit_length() - 1
        log_r = (len(c["codeword"]) // k).bit_length() - 1
        cw = O.encode_rows([num(x) for x in c["row"]], log_k, log_r, masks=[num(x) for x in c["mask"]],
                           mask_coeffs=c["mask_coeffs"])
        assert list(cw[0]) == [num(x) for x in c["codeword"]]


def test_streaming_commitments():
    for c in load("streaming")["cases"]:
        log_k = c["layout"]["log2_k"]
        k, n = 1 << log_k, len(c["leaves"])
        log_r = (n // k).bit_length() - 1
        rows = np.array([[num(x) for x in r] for r in c["rows"]], dtype=np.uint64).reshape(-1)
        masks = np.array([[num(x) for x in r] for r in c["masks"]], dtype=np.uint64).reshape(-1)
        nrows = len(c["rows"])
        cw = (O.encode_rows(rows, log_k, log_r, masks=masks, mask_coeffs=c["mask_coeffs"]) if nrows
              else np.zeros((0, n), dtype=np.uint64))
        for i in range(nrows):
            assert list(cw[i]) == [num(x) for x in c["codewords"][i]]
        cid = bytes.fromhex(c["commitment_id"])
        segs, off = [], 0
        for s, expected in zip(c["segments"], c["segment_digests"]):
            chains = O.column_chains(cid, cw[off:off + len(s)].reshape(-1), n, c["row_block"])
            assert [bytes(x).hex() for x in chains] == expected
            segs.append(chains)
            off += len(s)
        leaves, root = O.merge_segments(np.stack(segs))
        assert [bytes(x).hex() for x in leaves] == c["leaves"]
        assert root.hex() == c["root"]


def test_sumcheck_stages():
    v = load("sumcheck")
    seed = num(v["seed"])
    stages = 0
    for session in v["sessions"]:
        t = O.OracleTranscript(context_tce(session["context"]))
        for st in session["stages"]:
            tables = stage_tables(seed, st)
            insts = [[(tb, True, False) for tb in inst] for inst in tables]
            gamma, rounds, chal, evals = O.prove_batch(t, st["prefix"], st["degree"], insts)
            assert gamma == tuple(num(x) for x in st["gamma"])
            assert rounds == [fp2s(m) for m in st["rounds"]], (session["name"], st["prefix"])
            assert chal == fp2s(st["challenges"])
            assert evals == fp2s(st["final_evals"])
            assert t.state.hex() == st["state"] and t.counter == st["counter"]
            stages += 1
    assert stages == 62


def advice_stream(seed: bytes, words: int):
    raw = O.blake3("derive", seed, 8 * words, key="tessera/v1/advice-masks")
    return [int.from_bytes(raw[8 * i:8 * i + 8], "little") for i in range(words)]


def test_advice_mask_stream():
    """The advice mask stream (ProverDomain::AdviceMasks): the oracle's BLAKE3 extended output of
    H("advice-masks", seed), its words below p in order, reproduces the vectors' masks and the
    pinned seed whose word 6 is rejected."""
    ps = load("hash")["prover_streams"]
    words = advice_stream(bytes.fromhex(ps["proof_seed"]), 32)
    assert [w for w in words if w < P][:24] == [num(x) for x in ps["advice_masks"]]
    rj = ps["rejection"]
    words = advice_stream(bytes.fromhex(rj["seed"]), 16)
    assert words == [num(x) for x in rj["words"]] and words[rj["rejected_word_index"]] >= P
    assert [w for w in words if w < P] == [num(x) for x in rj["values"]]
