"""Serving with continuous batching: a proof server on the GPU (the C ABI's tg_server_*).

A request is one proof of the prover's shape: the resident unmasked commitment of its rows
(crates/tessera-pcs/src/commitment.rs:343-458), the root absorbed into the request's transcript
under "<prefix>/root", then a one-instance prove_batch of the product of its prime-field tables
under <prefix> (crates/tessera-sumcheck/src/prover.rs:1122), then, with `queries`, an opening round
on the commitment still resident on the device: indices drawn under "<prefix>/queries", the
queried columns and their canonical Merkle multiproof. Requests are admitted as stream slots and
HBM budget free up and overlap on the device; `prove_plain` is the same proof through the
one-call-at-a-time entry points, the plain path a served result must equal.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _native as N
from .device import Device, host_u64, resolve
from .hash import Transcript
from .pcs import CommitmentParams


@dataclass
class ProofRequest:
    params: CommitmentParams   # unmasked (mask_coeffs 0)
    rows: object               # host words, npolys x 2^log2_k (numpy uint64, or a pinned int64 tensor)
    degree: int
    tables: list               # host words, each 2^vars (prime-field tables)
    transcript: Transcript     # the proof's transcript at its start (not modified)
    prefix: str = "stage/0"
    queries: int = 0           # column queries answered after the proof


@dataclass
class ProofResult:
    root: bytes
    gamma: tuple[int, int]
    rounds: list[list[tuple[int, int]]]
    challenges: list[tuple[int, int]]
    final_evals: list[tuple[int, int]]
    state: bytes               # the transcript at the end of the proof
    counter: int
    queued_ms: float = 0.0
    latency_ms: float = 0.0
    stage_ms: tuple = ()        # when each stage (commit, sumcheck, opening) was seen to end, ms after submission
    query_indices: list = None  # the opening round: indices in draw order,
    columns: np.ndarray = None  # each distinct queried column's symbols (distinct x npolys, increasing index),
    siblings: list = None       # and the canonical multiproof of those indices

    def same_proof(self, other: "ProofResult") -> bool:
        mine = (self.root, self.gamma, self.rounds, self.challenges, self.final_evals, self.state, self.counter,
                self.query_indices, self.siblings)
        theirs = (other.root, other.gamma, other.rounds, other.challenges, other.final_evals, other.state,
                  other.counter, other.query_indices, other.siblings)
        same_cols = (self.columns is None and other.columns is None) or (
            self.columns is not None and other.columns is not None and np.array_equal(self.columns, other.columns))
        return mine == theirs and same_cols


def _words(x) -> np.ndarray:
    if hasattr(x, "numpy") and not getattr(x, "is_cuda", False):
        x = x.numpy()
    a = np.asarray(x)
    if a.dtype == np.int64:
        a = a.view(np.uint64)
    return host_u64(a).reshape(-1)


def _pairs(a, n):
    return [(int(a[2 * i]), int(a[2 * i + 1])) for i in range(n)]


class ProofServer:
    """Continuous batching on one GPU: `slots` requests in flight at most, admitted first come
    first served while their device memory fits `hbm_budget_bytes`."""

    def __init__(self, device: Device | None = None, hbm_budget_bytes: int = 64 << 30, slots: int = 8):
        self.device = resolve(device)
        self._srv = ctypes.c_void_p()
        N.call("tg_server_open", self.device.handle, hbm_budget_bytes, slots, ctypes.byref(self._srv))
        self._live = {}

    def submit(self, req: ProofRequest) -> int:
        p = req.params
        if p.mask_coeffs != 0:
            raise ValueError("served commitments are unmasked")
        rows = _words(req.rows)
        tabs = [_words(t) for t in req.tables]
        vars_ = max(len(tabs[0]), 1).bit_length() - 1 if tabs else 0
        c = N.ProofRequestC()
        c.log_k, c.log_inv_rate, c.row_block = p.log2_k, p.log2_inv_rate, p.row_block
        c.commitment_id[:] = list(bytes(p.commitment_id))
        c.rows = rows.ctypes.data if rows.size else None
        c.npolys = rows.size >> p.log2_k
        c.degree, c.ntables, c.vars = req.degree, len(tabs), vars_
        tptr = (ctypes.c_void_p * max(1, len(tabs)))(*[t.ctypes.data for t in tabs])
        c.tables = ctypes.cast(tptr, ctypes.POINTER(ctypes.c_void_p))
        c.transcript = req.transcript.raw
        pre = req.prefix.encode()
        c.prefix = pre
        c.queries = req.queries
        rounds = np.zeros(max(1, vars_ * req.degree * 2), dtype=np.uint64)
        chal = np.zeros(max(1, vars_ * 2), dtype=np.uint64)
        evals = np.zeros(max(1, len(tabs) * 2), dtype=np.uint64)
        out = N.ProofResultC()
        out.rounds, out.challenges, out.final_evals = rounds.ctypes.data, chal.ctypes.data, evals.ctypes.data
        log_n = p.log2_k + p.log2_inv_rate
        npolys = c.npolys
        qidx = np.zeros(max(1, req.queries), dtype=np.uint64)
        cols = np.zeros(max(1, req.queries * npolys), dtype=np.uint64)
        sibs = np.zeros(max(1, req.queries * log_n * 32), dtype=np.uint8)
        out.query_indices, out.columns, out.siblings = qidx.ctypes.data, cols.ctypes.data, sibs.ctypes.data
        ticket = ctypes.c_uint64()
        N.call("tg_server_submit", self._srv, ctypes.byref(c), ctypes.byref(out), ctypes.byref(ticket))
        # everything the request points at stays alive until it is collected
        self._live[ticket.value] = (c, out, rows, tabs, tptr, pre, rounds, chal, evals, req.degree, vars_,
                                    (req.queries, npolys, qidx, cols, sibs))
        return ticket.value

    def wait(self, ticket: int, timeout_ms: int = -1) -> ProofResult:
        N.call("tg_server_wait", self._srv, ticket, timeout_ms)
        c, out, rows, tabs, tptr, pre, rounds, chal, evals, degree, vars_, (tau, npolys, qidx, cols, sibs) = \
            self._live.pop(ticket)
        res = ProofResult(bytes(out.root), (int(out.gamma[0]), int(out.gamma[1])),
                          [_pairs(rounds[j * degree * 2:(j + 1) * degree * 2], degree) for j in range(vars_)],
                          _pairs(chal, vars_), _pairs(evals, len(tabs)), bytes(out.transcript.state),
                          int(out.transcript.counter), out.queued_ms, out.latency_ms, tuple(out.stage_ms))
        if tau:
            m, ns = out.n_distinct, out.n_siblings
            res.query_indices = [int(x) for x in qidx[:tau]]
            res.columns = cols[:m * npolys].reshape(m, npolys).copy()
            res.siblings = [bytes(sibs[32 * t:32 * t + 32]) for t in range(ns)]
        return res

    def stats(self) -> dict:
        st = N.ServerStatsC()
        N.call("tg_server_stats_read", self._srv, ctypes.byref(st))
        return {"submitted": st.submitted, "completed": st.completed, "peak_inflight": st.peak_inflight,
                "peak_bytes": st.peak_bytes}

    def close(self):
        if self._srv:
            N.call("tg_server_close", self._srv)
            self._srv = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def multiproof_nodes(n: int, indices) -> list[int]:
    """The node indices (leaves first, root last) of the canonical multiproof of `indices`: per
    level from the leaves up, the sibling of every opened node whose sibling is not opened, left to
    right (the order verifier/crates/tv-hash/src/merkle.rs:137-210 reads them in)."""
    out, base, width = [], 0, n
    cur = sorted(set(indices))
    while width > 1:
        s = set(cur)
        out.extend(base + (x ^ 1) for x in cur if x ^ 1 not in s)
        base += width
        width //= 2
        cur = sorted({x >> 1 for x in cur})
    return out


def prove_plain(req: ProofRequest, device: Device | None = None) -> ProofResult:
    """The same proof through the plain entry points, one call after another. With queries, the
    commitment is made device-resident (tg_commit_unmasked_dev) and answered from its codewords and
    Merkle nodes after the proof."""
    from .sumcheck import Instance, Protocol, Table, prove_batch

    d = resolve(device)
    p = req.params
    rows = _words(req.rows)
    npolys = rows.size >> p.log2_k
    # as the server does on submission: the host pages are touched before they are copied
    for x in [rows] + [_words(t) for t in req.tables]:
        if x.size:
            N.call("tg_host_prefault", ctypes.c_void_p(x.ctypes.data), x.nbytes)
    root = ctypes.create_string_buffer(32)
    cid = (ctypes.c_uint8 * 32)(*bytes(p.commitment_id))
    resident = None
    if req.queries:
        import torch

        n = 1 << (p.log2_k + p.log2_inv_rate)
        dev = f"cuda:{d.ordinal}"
        rows_d = torch.from_numpy(rows.view(np.int64)).to(dev)
        cw_d = torch.empty(npolys * n, dtype=torch.int64, device=dev)
        nodes_d = torch.empty((2 * n - 1) * 32, dtype=torch.uint8, device=dev)
        torch.cuda.current_stream().synchronize()
        N.call("tg_commit_unmasked_dev", d.handle, p.log2_k, p.log2_inv_rate, p.row_block, cid,
               ctypes.c_void_p(rows_d.data_ptr()), npolys, ctypes.c_void_p(cw_d.data_ptr()),
               ctypes.c_void_p(nodes_d.data_ptr()), root, None)
        resident = (n, cw_d, nodes_d)
    else:
        N.call("tg_commit_unmasked", d.handle, p.log2_k, p.log2_inv_rate, p.row_block, cid,
               ctypes.c_void_p(rows.ctypes.data) if rows.size else None, npolys, None, root)
    t = req.transcript.copy()
    t.absorb(req.prefix + "/root", root.raw)
    pb = prove_batch(t, Protocol.ONE, req.prefix, req.degree, [Instance([Table.base(_words(x)) for x in req.tables])],
                     device=d)
    res = ProofResult(root.raw, pb.gamma, pb.proof.rounds, pb.point, pb.proof.final_evals, t.state, t.counter)
    if resident:
        import torch

        n, cw_d, nodes_d = resident
        log_n = p.log2_k + p.log2_inv_rate
        res.query_indices = t.challenge_indices(req.prefix + "/queries", log_n, req.queries)
        distinct = sorted(set(res.query_indices))
        idx = torch.tensor(distinct, dtype=torch.int64, device=cw_d.device)
        res.columns = cw_d.view(npolys, n)[:, idx].t().contiguous().cpu().numpy().view(np.uint64)
        sel = torch.tensor(multiproof_nodes(n, distinct), dtype=torch.int64, device=cw_d.device)
        res.siblings = [bytes(x) for x in nodes_d.view(-1, 32)[sel].cpu().numpy()]
        res.state, res.counter = t.state, t.counter
    return res
