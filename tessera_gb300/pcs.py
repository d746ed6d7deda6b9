"""Commitments on the GPU: the reference's tessera-pcs surface for the hot path
(crates/tessera-pcs/src/lib.rs:352-375).

`NttPlan` (ntt.rs:461-516), `RowEncoder` (encoding.rs:126-313), `CommitmentParams` (commitment.rs:79-105),
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
from .device import Device, digests, host_u64, is_device_tensor, ptr, resolve, torch_stream

COSET_SHIFT = 7
P_FIELD = 0xFFFFFFFF00000001
Digest = bytes


def _log2_exact(n: int, what: str) -> int:
    if n < 1 or n & (n - 1):
        raise ValueError(f"{what} {n} is not a power of two")
    return n.bit_length() - 1


class NttPlan:
    """Transforms of size n = 2^log_size, natural order on both sides (the reference's NttPlan,
    crates/tessera-pcs/src/ntt.rs:461-516): ntt gives f(ω_n^j) from the coefficients, coset_ntt
    f(shift·ω_n^j), intt and coset_intt their inverses. Each takes one row of n values or many
    (an (m, n) array, or a flat array of whole rows): host arrays come back as new arrays, device
    tensors are transformed in place on torch's current stream."""

    def __init__(self, log_size: int, device: Device | None = None):
        if log_size > 22:
            raise ValueError(f"transforms of 2^{log_size} points: the device transforms go up to 2^22")
        self.log_size = log_size
        self.device = resolve(device)

    def size(self) -> int:
        return 1 << self.log_size

    def _run(self, name: str, values, shift=None):
        n = self.size()
        extra = [] if shift is None else [int(shift)]
        if shift is not None and (int(shift) % P_FIELD) == 0:
            raise ValueError("a coset shift of zero")
        if is_device_tensor(values):
            if values.numel() % n:
                raise ValueError(f"{values.numel()} values are not whole rows of {n}")
            N.call(f"tg_{name}_dev", self.device.handle, self.log_size, *extra, ctypes.c_void_p(values.data_ptr()),
                   values.numel() // n, torch_stream())
            return values
        v = np.array(host_u64(values), dtype=np.uint64, copy=True)
        if v.size % n:
            raise ValueError(f"{v.size} values are not whole rows of {n}")
        N.call(f"tg_{name}", self.device.handle, self.log_size, *extra, ptr(v), v.size // n)
        return v

    def ntt(self, values):
        return self._run("ntt", values)

    def intt(self, values):
        return self._run("intt", values)

    def coset_ntt(self, values, shift: int):
        return self._run("coset_ntt", values, shift)

    def coset_intt(self, values, shift: int):
        return self._run("coset_intt", values, shift)


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


# ---- the batched pattern: many commitments at once ---------------------------------------------

class ResidentCommitment:
    """One commitment of a batch, kept on the device: codewords (npolys x n words), nodes
    ((2n − 1) x 32 bytes, leaves first, root last) and the root."""

    def __init__(self, params: CommitmentParams, rows, codewords, nodes):
        self.params, self.rows, self.codewords, self.nodes = params, rows, codewords, nodes
        self.root: Digest = b""

    @property
    def npolys(self) -> int:
        return self.rows.numel() >> self.params.log2_k

    def leaves(self) -> list[Digest]:
        n = 1 << (self.params.log2_k + self.params.log2_inv_rate)
        return digests(self.nodes[: 32 * n].cpu().numpy().reshape(n, 32))


def _resident(params_list, rows_list, device: Device):
    import torch

    if len(params_list) != len(rows_list):
        raise ValueError("one row tensor per commitment")
    out = []
    arr = (N.CommitJobC * len(params_list))()
    for i, (p, rows) in enumerate(zip(params_list, rows_list)):
        if p.mask_coeffs != 0:
            raise ValueError("the batched commitments are unmasked")
        if not (hasattr(rows, "is_cuda") and rows.is_cuda):
            raise ValueError("the batched path takes rows already on the device (torch CUDA tensors)")
        k, n = 1 << p.log2_k, 1 << (p.log2_k + p.log2_inv_rate)
        if rows.numel() % k:
            raise ValueError(f"{rows.numel()} values are not whole rows of {k}")
        npolys = rows.numel() // k
        cw = torch.empty(max(npolys * n, 1), dtype=torch.int64, device=rows.device)
        nodes = torch.empty((2 * n - 1) * 32, dtype=torch.uint8, device=rows.device)
        rc = ResidentCommitment(p, rows, cw, nodes)
        out.append(rc)
        arr[i].log_k, arr[i].log_inv_rate, arr[i].row_block = p.log2_k, p.log2_inv_rate, p.row_block
        arr[i].commitment_id[:] = list(bytes(p.commitment_id))
        arr[i].rows = rows.data_ptr()
        arr[i].npolys = npolys
        arr[i].codewords = cw.data_ptr()
        arr[i].nodes = nodes.data_ptr()
    return out, arr


def commit_many(params_list: list[CommitmentParams], rows_list, device: Device | None = None,
                workers: int = 0) -> list[ResidentCommitment]:
    """Commits many unmasked batches of rows (device tensors, npolys x k words each) together on
    `workers` streams; each result equals `commit_unmasked` of the same rows."""
    import torch

    d = resolve(device)
    out, arr = _resident(params_list, rows_list, d)
    torch.cuda.current_stream().synchronize()
    N.call("tg_commit_many", d.handle, arr, len(out), workers)
    for i, rc in enumerate(out):
        rc.root = bytes(arr[i].root)
    return out


class CommitPlan:
    """A batch of commitments captured into one CUDA graph: the shapes and device buffers are
    fixed when the plan is made (the worker count autotuned on the batch unless given), and
    every `launch()` re-commits whatever the row tensors hold then."""

    def __init__(self, params_list: list[CommitmentParams], rows_list, device: Device | None = None, workers: int = 0):
        import torch

        self.device = resolve(device)
        self.commitments, self._arr = _resident(params_list, rows_list, self.device)
        torch.cuda.current_stream().synchronize()
        self._plan = ctypes.c_void_p()
        N.call("tg_commit_plan_create", self.device.handle, self._arr, len(self.commitments), workers,
               ctypes.byref(self._plan))

    def launch(self) -> list[Digest]:
        import torch

        torch.cuda.current_stream().synchronize()
        roots = ctypes.create_string_buffer(32 * len(self.commitments))
        N.call("tg_commit_plan_launch", self._plan, roots)
        out = [roots.raw[32 * i: 32 * (i + 1)] for i in range(len(self.commitments))]
        for rc, r in zip(self.commitments, out):
            rc.root = r
        return out

    def info(self) -> dict:
        w, kern = ctypes.c_int(), ctypes.c_uint64()
        ms = (ctypes.c_double * 4)()
        N.call("tg_commit_plan_info", self._plan, ctypes.byref(w), ctypes.byref(kern), ms)
        count = ctypes.c_int()
        N.call("tg_commit_plan_tuning", self._plan, None, 0, ctypes.byref(count))
        shapes = (N.EncodeTuningC * max(count.value, 1))()
        N.call("tg_commit_plan_tuning", self._plan, shapes, count.value, ctypes.byref(count))
        return {"workers": w.value, "kernels_per_launch": kern.value,
                "tuned_ms": {c: ms[i] for i, c in enumerate((1, 2, 4, 8)) if ms[i] > 0},
                "encoder_shapes": [{"log_k": t.log_k, "log_inv_rate": t.log_inv_rate, "rows": t.npolys,
                                    "split_log": t.split_log, "group": t.group, "candidates": t.candidates,
                                    "ms_default": t.ms_default, "ms_tuned": t.ms_tuned,
                                    "from_cache": bool(t.from_cache)} for t in shapes[:count.value]]}

    def close(self):
        if self._plan:
            N.call("tg_commit_plan_destroy", self._plan)
            self._plan = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class ColumnSink:
    """The opening's column sink on the GPU (the reference's ColumnSink and its GPU ColumnsSink):
    `select` re-encodes a block of whole rows with their masks and returns each row's symbols at
    the sink's columns; `select_combining` also adds the block's combined rows Σ_r c[g][r]·row_r
    to sums kept on the device; `combined` adds those sums into the caller's rows and clears them."""

    def __init__(self, encoder: RowEncoder, block: int, columns, device: Device | None = None):
        self.device = resolve(device or encoder.device)
        self.k, self.P = encoder.message_len(), encoder.mask_coeffs()
        cols = host_u64(columns).reshape(-1)
        self.m = cols.size
        self._sink = ctypes.c_void_p()
        N.call("tg_column_sink_open", self.device.handle, encoder.log_k, encoder.log_inv_rate, self.P, block, ptr(cols),
               cols.size, ctypes.byref(self._sink))

    def _rows(self, rows, masks):
        r = host_u64(rows).reshape(-1)
        if r.size % self.k:
            raise ValueError(f"{r.size} values are not whole rows of {self.k}")
        nrows = r.size // self.k
        m = host_u64(masks).reshape(-1) if self.P else None
        if self.P and (m is None or m.size != nrows * self.P):
            raise ValueError(f"expected {nrows * self.P} mask coefficients")
        return r, nrows, m

    def select(self, rows, masks=None) -> np.ndarray:
        r, nrows, m = self._rows(rows, masks)
        out = np.empty((nrows, self.m), dtype=np.uint64)
        N.call("tg_column_sink_select", self._sink, ptr(r), nrows, ptr(m), ptr(out))
        return out

    def combines(self) -> bool:
        return True

    def select_combining(self, rows, masks, coefficients) -> np.ndarray:
        """coefficients: one list per group of this block's row coefficients, each an Fp2 (c0, c1)."""
        r, nrows, m = self._rows(rows, masks)
        c = host_u64([w for grp in coefficients for pair in grp for w in pair])
        if c.size != 2 * nrows * len(coefficients):
            raise ValueError("one coefficient per row in every group")
        out = np.empty((nrows, self.m), dtype=np.uint64)
        N.call("tg_column_sink_select_combining", self._sink, ptr(r), nrows, ptr(m), ptr(c), len(coefficients), ptr(out))
        return out

    def combined(self, out: np.ndarray) -> np.ndarray:
        """Adds the sums into `out` (groups x k x 2 words, Fp2 pairs) in place and returns it."""
        o = np.ascontiguousarray(out, dtype=np.uint64)
        N.call("tg_column_sink_combined", self._sink, ptr(o), o.shape[0] if o.ndim == 3 else 0)
        if o is not out:
            out[...] = o
        return out

    def close(self):
        if self._sink:
            N.call("tg_column_sink_close", self._sink)
            self._sink = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
