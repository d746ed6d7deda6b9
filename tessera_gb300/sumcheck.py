"""Batched sumcheck on the GPU: the reference's prove_batch surface
(crates/tessera-sumcheck/src/prover.rs:1122-1421; Table :118-240, Instance :259-330, Prefix
:40-75, SumcheckProof in proof.rs:15-23).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np

from . import _native as N
from .device import Device, host_u64, is_device_tensor, ptr, resolve
from .hash import Transcript


class Prefix:
    """stage/{k}, tree/{l}, group/{h}/tree/{l}, tables/tree/{l}, merge (prover.rs:63-75)."""

    def __init__(self, text: str):
        self.text = text

    @classmethod
    def stage(cls, k: int) -> "Prefix":
        return cls(f"stage/{k}")

    @classmethod
    def tree(cls, level: int) -> "Prefix":
        return cls(f"tree/{level}")

    def __str__(self):
        return self.text


class Protocol:
    ONE = 1  # degrees 1..7


class Table:
    """A factor: 2^n entries over the prime field (`base`) or Fp2 (`ext`, interleaved c0, c1
    words, or an (m, 2) array); `public()` leaves its evaluation out of the proof."""

    def __init__(self, values, is_ext: bool, is_public: bool = False):
        self.is_ext, self.is_public = is_ext, is_public
        if is_device_tensor(values):
            self.device_values = values
            self.values = None
            self.len = values.numel() // (2 if is_ext else 1)
        else:
            self.device_values = None
            self.values = host_u64(values).reshape(-1)
            self.len = self.values.size // (2 if is_ext else 1)

    @classmethod
    def base(cls, values) -> "Table":
        return cls(values, False)

    @classmethod
    def ext(cls, values) -> "Table":
        return cls(values, True)

    def public(self) -> "Table":
        t = Table.__new__(Table)
        t.__dict__.update(self.__dict__)
        t.is_public = True
        return t


class Instance:
    """The product of its tables, all of 2^n entries."""

    def __init__(self, tables: list[Table]):
        self.tables = tables


@dataclass
class SumcheckProof:
    rounds: list[list[tuple[int, int]]]
    final_evals: list[tuple[int, int]]


@dataclass
class ProvenBatch:
    proof: SumcheckProof
    gamma: tuple[int, int]
    point: list[tuple[int, int]]
    vars: list[int] = field(default_factory=list)


def _pack(instances: list[Instance], keep: list, on_device=None):
    """The C view of a batch's instances: (tg_instance array, variables per instance, table count,
    whether the tables are device tensors)."""
    if not instances:
        raise N.InvalidInput(N.TG_ERR_INVALID, "a batch needs at least one instance")
    inst_arr = (N.InstanceC * len(instances))()
    vars_ = []
    ntables = 0
    for i, inst in enumerate(instances):
        if not inst.tables:
            raise N.InvalidInput(N.TG_ERR_INVALID, f"instance {i} has no table")
        lengths = {t.len for t in inst.tables}
        n0 = inst.tables[0].len
        if n0 < 1 or n0 & (n0 - 1):
            raise N.InvalidInput(N.TG_ERR_INVALID, f"instance {i}: table length {n0} is not a power of two")
        if len(lengths) != 1:
            raise N.InvalidInput(N.TG_ERR_INVALID, f"instance {i}: tables of different lengths {sorted(lengths)}")
        tarr = (N.TableC * len(inst.tables))()
        for k, t in enumerate(inst.tables):
            dev = t.device_values is not None
            if on_device is None:
                on_device = dev
            elif on_device != dev:
                raise ValueError("a batch's tables are all in host memory or all on the device")
            tarr[k].values = t.device_values.data_ptr() if dev else t.values.ctypes.data
            tarr[k].is_ext = int(t.is_ext)
            tarr[k].is_public = int(t.is_public)
            keep.append(t)
            ntables += 1
        keep.append(tarr)
        inst_arr[i].tables = ctypes.cast(tarr, ctypes.POINTER(N.TableC))
        inst_arr[i].ntables = len(inst.tables)
        inst_arr[i].vars = n0.bit_length() - 1
        vars_.append(n0.bit_length() - 1)
    keep.append(inst_arr)
    return inst_arr, vars_, ntables, on_device


def _pairs(a, n):
    return [(int(a[2 * i]), int(a[2 * i + 1])) for i in range(n)]


def _sync_torch(on_device):
    if on_device:
        import torch

        torch.cuda.current_stream().synchronize()


def prove_batch(transcript: Transcript, protocol: int, prefix, degree: int, instances: list[Instance],
                device: Device | None = None) -> ProvenBatch:
    """Proves Σ_i γ^i·P_i over the front-padded hypercube; the transcript advances exactly as
    the reference's."""
    d = resolve(device)
    keep = []
    inst_arr, vars_, evals_cap, on_device = _pack(instances, keep)
    n_max = max(vars_)
    gamma = (ctypes.c_uint64 * 2)()
    rounds = np.zeros(max(1, n_max * degree * 2), dtype=np.uint64)
    chal = np.zeros(max(1, n_max * 2), dtype=np.uint64)
    evals = np.zeros(max(1, evals_cap * 2), dtype=np.uint64)
    ne = ctypes.c_size_t()
    _sync_torch(on_device)
    N.call("tg_prove_batch", d.handle, ctypes.byref(transcript.raw), str(prefix).encode(), degree, inst_arr,
           len(instances), int(bool(on_device)), gamma, ptr(rounds), ptr(chal), ptr(evals), ctypes.byref(ne))
    rr = [_pairs(rounds[j * degree * 2:(j + 1) * degree * 2], degree) for j in range(n_max)]
    return ProvenBatch(SumcheckProof(rr, _pairs(evals, ne.value)), (int(gamma[0]), int(gamma[1])), _pairs(chal, n_max),
                       vars_)


def prove_many(jobs: list[tuple[Transcript, int, object, int, list[Instance]]],
               device: Device | None = None) -> list[ProvenBatch]:
    """Many independent prove_batch calls, each (transcript, protocol, prefix, degree, instances)
    with its own transcript, proved together: one fused launch per round for all jobs and one for
    all their transcripts. Equal, byte for byte, to calling prove_batch on each job in turn."""
    d = resolve(device)
    if not jobs:
        raise N.InvalidInput(N.TG_ERR_INVALID, "no sumcheck jobs")
    keep = []
    arr = (N.SumcheckJobC * len(jobs))()
    outs = []
    on_device = None
    for b, (transcript, _protocol, prefix, degree, instances) in enumerate(jobs):
        inst_arr, vars_, ntables, on_device = _pack(instances, keep, on_device)
        n_max = max(vars_)
        rounds = np.zeros(max(1, n_max * degree * 2), dtype=np.uint64)
        chal = np.zeros(max(1, n_max * 2), dtype=np.uint64)
        evals = np.zeros(max(1, ntables * 2), dtype=np.uint64)
        pre = str(prefix).encode()
        keep.extend([rounds, chal, evals, pre])
        arr[b].transcript = ctypes.addressof(transcript.raw)
        arr[b].prefix = pre
        arr[b].degree = degree
        arr[b].instances = ctypes.cast(inst_arr, ctypes.POINTER(N.InstanceC))
        arr[b].ninstances = len(instances)
        arr[b].rounds = rounds.ctypes.data
        arr[b].challenges = chal.ctypes.data
        arr[b].final_evals = evals.ctypes.data
        outs.append((degree, n_max, vars_, rounds, chal, evals))
    _sync_torch(on_device)
    N.call("tg_prove_many", d.handle, arr, len(jobs), int(bool(on_device)))
    res = []
    for b, (degree, n_max, vars_, rounds, chal, evals) in enumerate(outs):
        rr = [_pairs(rounds[j * degree * 2:(j + 1) * degree * 2], degree) for j in range(n_max)]
        res.append(ProvenBatch(SumcheckProof(rr, _pairs(evals, arr[b].n_evals)),
                               (int(arr[b].gamma[0]), int(arr[b].gamma[1])), _pairs(chal, n_max), vars_))
    return res
