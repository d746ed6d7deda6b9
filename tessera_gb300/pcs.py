"""Commitments on the GPU: the reference's tessera-pcs surface for the hot path
(crates/tessera-pcs/src/lib.rs:352-375).

`RowEncoder` (encoding.rs:126-313), `CommitmentParams` (commitment.rs:79-105),
`ReferenceCommitment.commit_unmasked` (commitment.rs:343-458), the `BlockSink` that
`StreamingCommitter::with_sink` drives (streaming.rs:24-37, the reference's AdviceSink),
`merge_segments` (streaming.rs:382-404), and `WeightEncoding`/`MatrixSink`
(weights/regenerated.rs:24-58). Host arrays in, host results out; the device-resident forms are
the `*_dev` entry points of the C ABI.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _native as N
from .device import Device, digests, host_u64, ptr, resolve

COSET_SHIFT = 7
Digest = bytes


def _log2_exact(n: int, what: str) -> int:
    if n < 1 or n & (n - 1):
        raise ValueError(f"{what} {n} is not a power of two")
    return n.bit_length() - 1


class RowEncoder:
    """Encodes rows of k values into codewords of n = 2^r k symbols with P mask coefficients:
    symbol j is g(7 ω_n^j), g = f + (X^k − 1) m."""

    def __init__(self, message_len: int, log2_inv_rate: int, mask_coeffs: int = 0, device: Device | None = None):
        self.log_k = _log2_exact(message_len, "message length")
        if log2_inv_rate == 0:
            raise ValueError("log2 inverse rate 0 is a code of rate 1")
        if self.log_k + log2_inv_rate > 32:
            raise ValueError(f"a codeword of 2^{self.log_k + log2_inv_rate} points exceeds 2^32")
        if mask_coeffs > message_len:
            raise ValueError(f"{mask_coeffs} mask coefficients exceed k = {message_len}")
        self.log_inv_rate = log2_inv_rate
        self.mask_coeffs_ = mask_coeffs
        self.device = resolve(device)

    def message_len(self) -> int:
        return 1 << self.log_k

    def codeword_len(self) -> int:
        return 1 << (self.log_k + self.log_inv_rate)

    def mask_coeffs(self) -> int:
        return self.mask_coeffs_

    def encode_rows(self, rows, masks=None) -> np.ndarray:
        """rows: nrows x k values (row-major); masks: nrows x P coefficients, m_0 first."""
        k, n, P = self.message_len(), self.codeword_len(), self.mask_coeffs_
        r = host_u64(rows).reshape(-1)
        if r.size % k:
            raise ValueError(f"{r.size} values are not whole rows of {k}")
        nrows = r.size // k
        m = host_u64(masks).reshape(-1) if P else None
        if P and (m is None or m.size != nrows * P):
            raise ValueError(f"expected {nrows * P} mask coefficients")
        out = np.empty((nrows, n), dtype=np.uint64)
        N.call("tg_encode_rows", self.device.handle, self.log_k, self.log_inv_rate, P, ptr(r), nrows, ptr(m), ptr(out))
        return out

    def encode_row(self, row, masks=None) -> np.ndarray:
        return self.encode_rows(row, masks)[0]


@dataclass
class CommitmentParams:
    log2_k: int
    log2_inv_rate: int
    mask_coeffs: int
    row_block: int
    commitment_id: Digest


class ReferenceCommitment:
    """The resident commitment: codewords encoded, one chain per column, Merkle root."""

    def __init__(self, params: CommitmentParams, leaves: list[Digest], root: Digest):
        self.params, self._leaves, self._root = params, leaves, root

    @classmethod
    def commit_unmasked(cls, params: CommitmentParams, rows, device: Device | None = None) -> "ReferenceCommitment":
        """Unmasked rows (P = 0) of one segment: leaf_j is the column's last chain digest."""
        if params.mask_coeffs != 0:
            raise ValueError("commit_unmasked takes no mask coefficients")
        d = resolve(device)
        k = 1 << params.log2_k
        r = host_u64(rows).reshape(-1)
        if r.size % k:
            raise ValueError(f"{r.size} values are not whole rows of {k}")
        n = k << params.log2_inv_rate
        leaves = np.zeros((n, 32), dtype=np.uint8)
        root = ctypes.create_string_buffer(32)
        cid = np.frombuffer(bytes(params.commitment_id), dtype=np.uint8).copy()
        N.call("tg_commit_unmasked", d.handle, params.log2_k, params.log2_inv_rate, params.row_block, ptr(cid), ptr(r),
               r.size // k, ptr(leaves), root)
        return cls(params, digests(leaves), root.raw)

    def root(self) -> Digest:
        return self._root

    def leaves(self) -> list[Digest]:
        return self._leaves


class AdviceSink:
    """A BlockSink on the GPU (the reference's AdviceSink): each absorb encodes one block of
    whole rows with their masks and absorbs the codewords into every column chain."""

    def __init__(self, params: CommitmentParams, device: Device | None = None):
        self.device = resolve(device)
        self.params = params
        self.k = 1 << params.log2_k
        self.n = self.k << params.log2_inv_rate
        h = ctypes.c_void_p()
        cid = np.frombuffer(bytes(params.commitment_id), dtype=np.uint8).copy()
        N.call("tg_advice_sink_open", self.device.handle, params.log2_k, params.log2_inv_rate, params.mask_coeffs,
               params.row_block, ptr(cid), ctypes.byref(h))
        self._h = h

    def absorb(self, rows, masks):
        r = host_u64(rows).reshape(-1)
        m = host_u64(masks).reshape(-1) if self.params.mask_coeffs else None
        if r.size % self.k:
            raise ValueError(f"{r.size} values are not whole rows of {self.k}")
        N.call("tg_sink_absorb", self._h, ptr(r), r.size // self.k, ptr(m))

    def finish(self) -> list[Digest]:
        out = np.zeros((self.n, 32), dtype=np.uint8)
        N.call("tg_sink_finish", self._h, ptr(out))
        return digests(out)

    def close(self):
        if self._h:
            N.lib().tg_sink_close(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass
class AdviceCommitment:
    root: Digest
    leaves: list[Digest]


def merge_segments(parts: list[list[Digest]], device: Device | None = None) -> AdviceCommitment:
    """Every leaf hashes all segments' digests in order: H("column-merge", d_j^(1) ‖ …)."""
    if not parts:
        raise ValueError("merge_segments needs at least one segment")
    n = len(parts[0])
    if any(len(p) != n for p in parts):
        raise ValueError("segments of different column counts")
    d = resolve(device)
    seg = np.frombuffer(b"".join(bytes(x) for p in parts for x in p), dtype=np.uint8).copy()
    leaves = np.zeros((n, 32), dtype=np.uint8)
    root = ctypes.create_string_buffer(32)
    N.call("tg_merge_segments", d.handle, ptr(seg), len(parts), n, ptr(leaves), root)
    return AdviceCommitment(root.raw, digests(leaves))


class MatrixSink:
    """One weight matrix encoded on the GPU: absorb returns each row's queried symbols."""

    def __init__(self, device: Device, log_k: int, log2_inv_rate: int, block: int, commitment_id: Digest, queries):
        self.device = device
        self.k = 1 << log_k
        self.n = self.k << log2_inv_rate
        self.q = host_u64(queries).reshape(-1)
        h = ctypes.c_void_p()
        cid = np.frombuffer(bytes(commitment_id), dtype=np.uint8).copy()
        N.call("tg_matrix_open", device.handle, log_k, log2_inv_rate, block, ptr(cid), ptr(self.q), self.q.size,
               ctypes.byref(h))
        self._h = h

    def absorb(self, rows) -> np.ndarray:
        r = host_u64(rows).reshape(-1)
        nrows = r.size // self.k
        out = np.zeros(max(1, nrows * self.q.size), dtype=np.uint64)
        N.call("tg_matrix_absorb", self._h, ptr(r), nrows, ptr(out))
        return out[: nrows * self.q.size]

    def finish(self) -> list[Digest]:
        out = np.zeros((self.n, 32), dtype=np.uint8)
        N.call("tg_matrix_finish", self._h, ptr(out))
        return digests(out)

    def close(self):
        if self._h:
            N.lib().tg_matrix_close(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class GpuWeights:
    """WeightEncoding on the GPU: opens a MatrixSink for any rate 1/2^r with r in 1..4."""

    def __init__(self, device: Device | None = None):
        self.device = resolve(device)

    def matrix(self, log_k: int, log2_inv_rate: int, block: int, commitment_id: Digest, columns: int, queries):
        if columns != 1 << (log_k + log2_inv_rate) or not 1 <= log2_inv_rate <= 4 or log_k > 24 or not 1 <= block <= 124:
            return None  # declined: the host encodes
        return MatrixSink(self.device, log_k, log2_inv_rate, block, commitment_id, queries)
