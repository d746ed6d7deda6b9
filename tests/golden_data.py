"""Loaders for the committed golden fixtures (tests/golden/*.json.gz), which hold the reference's
conformance vectors, and helpers to rebuild their inputs."""
from __future__ import annotations

import functools
import gzip
import json
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"
P = 0xFFFFFFFF00000001
MASK64 = (1 << 64) - 1


@functools.lru_cache(maxsize=None)
def load(name: str):
    with gzip.open(GOLDEN / f"{name}.json.gz", "rb") as f:
        return json.loads(f.read())


def num(x) -> int:
    """A vector's number: "0x.." hex or a decimal string."""
    if isinstance(x, int):
        return x
    return int(x, 16) if x.startswith("0x") else int(x)


def fp2s(values):
    return [(num(a), num(b)) for a, b in values]


def context_tce(ctx: dict) -> bytes:
    """TCE(SessionContext): u64-length-prefixed protocol, u16 mode tag, u64-length-prefixed
    params, statement digest, session id (tessera-hash/src/transcript.rs SessionContext)."""
    le = lambda n, b=8: n.to_bytes(b, "little")
    p, q = ctx["protocol"].encode(), ctx["params"].encode()
    mode = {"Live": 0, "NonInteractive": 1}[ctx["mode"]]
    return le(len(p)) + p + le(mode, 2) + le(len(q)) + q + bytes.fromhex(ctx["statement_digest"]) + bytes.fromhex(ctx["session_id"])


def splitmix64(state: int):
    while True:
        state = (state + 0x9E3779B97F4A7C15) & MASK64
        z = state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK64
        yield z ^ (z >> 31)


def stage_tables(seed: int, stage: dict):
    """The stage's tables, regenerated from the reference oracle's stream: each instance's
    tables, each 2^vars Fp2 entries drawn as two words below P (words at or above P rejected),
    starting `table_word_offset` words into SplitMix64(seed). Returns a list per instance of
    numpy arrays of interleaved (c0, c1) words."""
    rng = splitmix64(seed)
    for _ in range(stage["table_word_offset"]):
        next(rng)

    def fp():
        while True:
            x = next(rng)
            if x < P:
                return x

    out = []
    for inst in stage["instances"]:
        n, k = inst["vars"], inst["factors"]
        tables = []
        for _ in range(k):
            words = np.empty(2 << n, dtype=np.uint64)
            for i in range(2 << n):
                words[i] = fp()
            tables.append(words)
        out.append(tables)
    return out


def blake3_input(n: int) -> bytes:
    return bytes(i % 251 for i in range(n))
