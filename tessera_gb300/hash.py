"""Hashing and Fiat–Shamir: the reference's tessera-hash surface (crates/tessera-hash/src/lib.rs).

`hash`/`Domain` (domain.rs:41-181), `ColumnChains` (columns.rs:72-146), `MerkleTree` and
`merkle_node` (merkle.rs:10-117), `SessionContext`, `Mode` and `Transcript`
(transcript.rs:1-250). Column chains and trees run on the GPU; the transcript runs in the
library's host code.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _native as N
from .device import Device, digests, host_u64, ptr, resolve, torch_stream

Digest = bytes


def hash(domain: str, data: bytes) -> Digest:  # noqa: A001 - the reference's name
    """H(domain, data) = BLAKE3 derive-key("tessera/v1/" + domain, data)."""
    out = ctypes.create_string_buffer(32)
    buf = ctypes.create_string_buffer(bytes(data), max(1, len(data)))
    N.call("tg_hash", domain.encode(), buf, len(data), out)
    return out.raw


def merkle_node(left: Digest, right: Digest) -> Digest:
    return hash("merkle-node", bytes(left) + bytes(right))


class Mode:
    LIVE = 0
    NON_INTERACTIVE = 1


def _ascii(s: str) -> bytes:
    b = s.encode("ascii")
    return len(b).to_bytes(8, "little") + b


@dataclass
class SessionContext:
    protocol: str
    mode: int
    params: str
    statement_digest: bytes
    session_id: bytes

    def tce(self) -> bytes:
        """TCE(SessionContext): Ascii protocol, u16 mode tag, Ascii params, digest, session id."""
        if len(self.statement_digest) != 32 or len(self.session_id) != 16:
            raise ValueError("a statement digest is 32 bytes and a session id 16")
        return (_ascii(self.protocol) + int(self.mode).to_bytes(2, "little") + _ascii(self.params)
                + bytes(self.statement_digest) + bytes(self.session_id))


class Transcript:
    """The reference's Transcript: a 32-byte state and a squeeze counter."""

    def __init__(self, context: SessionContext | bytes):
        self._t = N.TranscriptState()
        tce = context.tce() if isinstance(context, SessionContext) else bytes(context)
        buf = ctypes.create_string_buffer(tce, max(1, len(tce)))
        N.call("tg_transcript_init", ctypes.byref(self._t), buf, len(tce))

    @classmethod
    def from_state(cls, state: bytes, counter: int) -> "Transcript":
        """A transcript resumed at a known state (as a fork of a proof's transcript)."""
        t = cls.__new__(cls)
        t._t = N.TranscriptState()
        t._t.state[:] = list(bytes(state))
        t._t.counter = counter
        return t

    def copy(self) -> "Transcript":
        return Transcript.from_state(self.state, self.counter)

    @property
    def state(self) -> Digest:
        return bytes(self._t.state)

    @property
    def counter(self) -> int:
        return int(self._t.counter)

    def absorb(self, label: str, value: bytes):
        buf = ctypes.create_string_buffer(bytes(value), max(1, len(value)))
        N.call("tg_transcript_absorb", ctypes.byref(self._t), label.encode(), buf, len(value))

    def absorb_fp2s(self, label: str, values):
        """Absorbs TCE Vec<Fp2> (sumcheck/src/transcript.rs:35-44)."""
        a = host_u64([w for v in values for w in v]) if len(values) else np.zeros(2, dtype=np.uint64)
        N.call("tg_transcript_absorb_fp2s", ctypes.byref(self._t), label.encode(), ptr(a), len(values))

    def squeeze(self, label: str) -> Digest:
        out = ctypes.create_string_buffer(32)
        N.call("tg_transcript_squeeze", ctypes.byref(self._t), label.encode(), out)
        return out.raw

    def challenge_fp(self, label: str) -> int:
        out = ctypes.c_uint64()
        N.call("tg_transcript_challenge_fp", ctypes.byref(self._t), label.encode(), ctypes.byref(out))
        return out.value

    def challenge_fp2(self, label: str) -> tuple[int, int]:
        out = (ctypes.c_uint64 * 2)()
        N.call("tg_transcript_challenge_fp2", ctypes.byref(self._t), label.encode(), out)
        return (int(out[0]), int(out[1]))

    def challenge_indices(self, label: str, log_n: int, count: int) -> list[int]:
        out = (ctypes.c_uint64 * max(1, count))()
        N.call("tg_transcript_challenge_indices", ctypes.byref(self._t), label.encode(), log_n, count, out)
        return [int(out[i]) for i in range(count)]

    def grind(self, label: str, bits: int, device: Device | None = None) -> int:
        """The smallest nonce whose H("pow", state ‖ label ‖ nonce) has `bits` leading zero
        bits, searched on the GPU, then absorbed (transcript.rs:241-250)."""
        d = resolve(device)
        out = ctypes.c_uint64()
        N.call("tg_transcript_grind", d.handle, ctypes.byref(self._t), label.encode(), bits, ctypes.byref(out))
        return out.value

    def check_grind(self, label: str, bits: int, nonce: int) -> bool:
        valid = ctypes.c_int()
        N.call("tg_transcript_check_grind", ctypes.byref(self._t), label.encode(), bits, nonce, ctypes.byref(valid))
        return bool(valid.value)

    # for the sumcheck driver
    @property
    def raw(self):
        return self._t


class ColumnChains:
    """Chained column digests on the GPU: d_j[0] = H("column-init", id ‖ u64 j), then one
    H("column-step", d_j ‖ symbols) per block of rows."""

    def __init__(self, commitment_id: Digest, columns: int, block: int, device: Device | None = None):
        import torch  # device memory only

        if columns < 1 or block < 1:
            raise ValueError("a commitment has at least one column and a block of at least one row")
        self.device = resolve(device)
        self.columns, self.block, self.closed = columns, block, False
        self._chains = torch.empty(columns * 32, dtype=torch.uint8, device=f"cuda:{self.device.ordinal}")
        cid = np.frombuffer(bytes(commitment_id), dtype=np.uint8).copy()
        N.call("tg_column_init_dev", self.device.handle, ptr(cid), columns, ctypes.c_void_p(self._chains.data_ptr()),
               torch_stream())

    def absorb_block(self, rows):
        """The next block, row-major: `block` whole rows, or fewer for the last block."""
        import torch

        rows = host_u64(rows).reshape(-1)
        if self.closed:
            raise N.TesseraError(N.TG_ERR_STATE, "a block followed the short final block")
        if rows.size % self.columns:
            raise ValueError(f"{rows.size} symbols do not fill rows of {self.columns} columns")
        count = rows.size // self.columns
        if count == 0 or count > self.block:
            raise ValueError(f"a block holds 1 to {self.block} rows, not {count}")
        d = torch.from_numpy(rows.view(np.int64)).to(f"cuda:{self.device.ordinal}")
        N.call("tg_column_absorb_dev", self.device.handle, ctypes.c_void_p(self._chains.data_ptr()), self.columns,
               ctypes.c_void_p(d.data_ptr()), count, self.block, torch_stream())
        self.closed = count < self.block

    def finish(self) -> list[Digest]:
        return digests(self._chains.cpu().numpy())


class MerkleTree:
    """A binary Merkle tree over a power-of-two number of leaves, built on the GPU; every level
    is kept, leaves first (merkle.rs:93-113)."""

    def __init__(self, leaves, device: Device | None = None):
        import torch

        lv = np.ascontiguousarray(np.frombuffer(b"".join(bytes(x) for x in leaves), dtype=np.uint8)
                                  if isinstance(leaves, (list, tuple)) else np.asarray(leaves, dtype=np.uint8)).reshape(-1, 32)
        n = lv.shape[0]
        if n == 0 or n & (n - 1):
            raise ValueError(f"a Merkle tree needs a power-of-two number of leaves, not {n}")
        d = resolve(device)
        dev = f"cuda:{d.ordinal}"
        src = torch.from_numpy(np.array(lv.reshape(-1), copy=True)).to(dev)
        nodes = torch.empty((2 * n - 1) * 32, dtype=torch.uint8, device=dev)
        N.call("tg_merkle_tree_dev", d.handle, ctypes.c_void_p(src.data_ptr()), n, ctypes.c_void_p(nodes.data_ptr()),
               torch_stream())
        self._nodes = nodes.cpu().numpy().reshape(-1, 32)
        self._leaves = n

    def root(self) -> Digest:
        return bytes(self._nodes[-1])

    def leaves(self) -> int:
        return self._leaves

    def nodes(self) -> np.ndarray:
        return self._nodes


def advice_masks(seed: bytes, count: int, first: int = 0, device: Device | None = None) -> np.ndarray:
    """The advice mask stream of `seed` (ProverDomain::AdviceMasks, crates/tessera-hash/src/
    domain.rs:83-127): values first .. first + count of the words below p of BLAKE3's extended
    output of H("advice-masks", seed), computed on the GPU."""
    d = resolve(device)
    out = np.zeros(max(1, count), dtype=np.uint64)
    buf = ctypes.create_string_buffer(bytes(seed), max(1, len(seed)))
    N.call("tg_advice_masks", d.handle, buf, len(seed), first, count, out.ctypes.data)
    return out[:count]
