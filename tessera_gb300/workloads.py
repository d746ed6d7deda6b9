"""Seeded synthetic workloads with the shapes of the reference benchmark's configurations: uniform
Goldilocks words from SplitMix64 (state += 0x9E3779B97F4A7C15, then the mix; words at or above p
reduced once, as `from_u64_reduced` does in crates/tessera-bench/benches/primitives.rs:52-69).

The batched workload is 64 commitments with row counts log-uniform in 2^10..2^20, polynomial counts
uniform in {8, 32, 128, 512} and rate 1/2 or 1/4, plus 64 sumchecks with variable counts uniform in
10..22 and degree 2 or 3, each sumcheck on its own transcript (session id = its index, little
endian). Every draw comes from one SplitMix64 stream started at the seed."""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

P = 0xFFFFFFFF00000001
GOLDEN = 0x9E3779B97F4A7C15


def splitmix_words(seed: int, n: int) -> np.ndarray:
    """n uniform Goldilocks words: SplitMix64 from `seed`, each output reduced below p."""
    out = np.empty(n, dtype=np.uint64)
    chunk = 1 << 24
    golden = np.uint64(GOLDEN)
    with np.errstate(over="ignore"):
        for s in range(0, n, chunk):
            m = min(chunk, n - s)
            z = (np.arange(s + 1, s + m + 1, dtype=np.uint64) * golden) + np.uint64(seed)
            z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
            z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
            z = z ^ (z >> np.uint64(31))
            out[s:s + m] = np.where(z >= np.uint64(P), z - np.uint64(P), z)
    return out


def fill_device(tensor, seed: int, device=None):
    """Fills an int64 CUDA tensor in place with splitmix_words(seed, numel), generated on the GPU."""
    from . import _native as N
    from .device import resolve

    d = resolve(device)
    N.call("tg_fill_splitmix", d.handle, tensor.data_ptr(), tensor.numel(), seed & (2**64 - 1), None)
    d.sync()
    return tensor


def counter_words(base: int, n: int) -> np.ndarray:
    """The reference's counter generator: word i is counter(base + i), the SplitMix64 output for
    state (base + i + 1)·0x9E3779B97F4A7C15 reduced once below p, i.e. the stream above started at
    base·0x9E3779B97F4A7C15."""
    return splitmix_words((base * GOLDEN) & (2**64 - 1), n)


def fill_counter(tensor, base: int, device=None):
    """Fills an int64 CUDA tensor in place with counter_words(base, numel), on the GPU (the
    reference's Device::fill_counter)."""
    from . import _native as N
    from .device import resolve

    d = resolve(device)
    N.call("tg_fill_counter", d.handle, tensor.data_ptr(), tensor.numel(), base & (2**64 - 1), None)
    d.sync()
    return tensor


class _Stream:
    def __init__(self, seed: int):
        self.state = seed & (2**64 - 1)

    def next(self) -> int:
        self.state = (self.state + GOLDEN) & (2**64 - 1)
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & (2**64 - 1)
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & (2**64 - 1)
        return z ^ (z >> 31)

    def below(self, n: int) -> int:
        return self.next() % n


@dataclass
class CommitShape:
    log_k: int
    polys: int
    log_inv_rate: int
    seed: int            # the rows' SplitMix64 seed
    commitment_id: bytes


@dataclass
class SumcheckShape:
    vars: int
    degree: int
    seed: int            # the tables' seed (table i from seed + i)
    session_id: bytes


def batched(seed: int, commitments: int = 64, sumchecks: int = 64, max_log_k: int = 20, max_polys: int = 512,
            max_vars: int = 22) -> tuple[list[CommitShape], list[SumcheckShape]]:
    """The batched workload's shapes. The caps shrink the draws for tests (a draw above a cap is
    clamped to it), leaving the sequence of draws unchanged."""
    st = _Stream(seed)
    cs = []
    for i in range(commitments):
        log_k = min(10 + st.below(11), max_log_k)
        polys = min((8, 32, 128, 512)[st.below(4)], max_polys)
        log_r = 1 + st.below(2)
        cid = b"".join(st.next().to_bytes(8, "little") for _ in range(4))
        cs.append(CommitShape(log_k, polys, log_r, st.next(), cid))
    ss = []
    for i in range(sumchecks):
        vars_ = min(10 + st.below(13), max_vars)
        degree = 2 + st.below(2)
        ss.append(SumcheckShape(vars_, degree, st.next(), i.to_bytes(16, "little")))
    return cs, ss
