"""Tree levels on the GPU: product forests and LogUp fraction trees, proven level by level from the
roots (RFC-0010 'Tree levels'; the reference's FractionTree, crates/tessera-sumcheck/src/trees.rs:260-345,
prove_trees :761, prove_forests, and LogUp's leaf stage, crates/tessera-logup/src/prover.rs:361).

Field elements are Fp2 pairs (c0, c1) of canonical words; tables are numpy uint64 arrays of
interleaved pairs (or device tensors with `on_device=True`)."""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np

from . import _native as N
from .device import Device, host_u64, is_device_tensor, resolve
from .hash import Transcript

P = 0xFFFFFFFF00000001


def lift(values) -> np.ndarray:
    """Prime-field words as Fp2 pairs (c1 = 0)."""
    v = host_u64(values).reshape(-1)
    out = np.zeros(2 * v.size, dtype=np.uint64)
    out[0::2] = v
    return out


def _entries(x) -> int:
    return x.numel() if hasattr(x, "numel") else np.asarray(x).size


@dataclass
class Forest:
    """2^s product trees of one height, from their stacked leaves: 2^(s+h) Fp2 entries, or
    prime-field words with `base` (the reference's GPU forest takes those, and keeps every level in
    the prime field)."""
    s: int
    leaves: np.ndarray
    base: bool = False

    @property
    def height(self) -> int:
        return (_entries(self.leaves) // (1 if self.base else 2)).bit_length() - 1 - self.s


@dataclass
class LeafGen:
    """Generated LogUp leaves (tg_leaf_gen): leaf j is (1 or −m_j, α − (k_j + β·v_j)) from the
    counter generator; mult_seed None: numerators of 1."""
    key_seed: int
    value_seed: int
    mult_seed: int | None
    alpha: tuple
    beta: tuple


@dataclass
class Fraction:
    """A LogUp fraction tree from its leaves' numerators (Fp2, or None for 1) and denominators.
    With `gen`, the leaf stage writes the generated leaves into these device tensors when it opens,
    in the same pass as the two levels above them."""
    denominators: np.ndarray
    numerators: np.ndarray | None = None
    sent: tuple | None = None  # the root (n, d) as the roots message carries it
    gen: LeafGen | None = None

    @property
    def height(self) -> int:
        return (_entries(self.denominators) // 2).bit_length() - 1


@dataclass
class LevelRecord:
    prefix: str
    root_challenges: list
    gamma: tuple
    lambda_: tuple | None
    rounds: list
    challenges: list
    claims: list
    final_evals: list
    rho: tuple
    present: list
    state: bytes = b""
    counter: int = 0


def _pairs(a, n):
    return [(int(a[2 * i]), int(a[2 * i + 1])) for i in range(n)]


class LeafStage:
    """The trees of one leaf stage in schedule order, their levels built on the device."""

    def __init__(self, trees: list, device: Device | None = None):
        self.device = resolve(device)
        self.trees = trees
        self._keep = []
        on_device = any(is_device_tensor(getattr(t, f, None)) for t in trees for f in ("leaves", "denominators"))

        def words(x):
            """The address of a table: a device tensor's, or a host copy's."""
            if on_device:
                if not is_device_tensor(x):
                    raise ValueError("a stage's leaves are all in host memory or all on the device")
                return x.data_ptr()
            a = host_u64(x).reshape(-1)
            self._keep.append(a)
            return a.ctypes.data

        arr = (N.TreeC * len(trees))()
        for k, t in enumerate(trees):
            if isinstance(t, Forest):
                arr[k].kind, arr[k].s, arr[k].height = 0, t.s, t.height
                arr[k].leaves = words(t.leaves)
                arr[k].base_leaves = int(t.base)
            else:
                arr[k].kind, arr[k].s, arr[k].height = 1, 0, t.height
                arr[k].denominators = words(t.denominators)
                if t.numerators is not None:
                    arr[k].leaves = words(t.numerators)
                if t.gen is not None:
                    g = t.gen
                    gc = N.LeafGenC(g.key_seed, g.value_seed, g.mult_seed or 0, int(g.mult_seed is None),
                                    (ctypes.c_uint64 * 2)(*g.alpha), (ctypes.c_uint64 * 2)(*g.beta))
                    self._keep.append(gc)
                    arr[k].gen = ctypes.addressof(gc)
                if t.sent is not None:
                    sent = host_u64([t.sent[0][0], t.sent[0][1], t.sent[1][0], t.sent[1][1]])
                    arr[k].sent = sent.ctypes.data
                    self._keep.append(sent)
        self._h = ctypes.c_void_p()
        if on_device:
            import torch

            torch.cuda.current_stream().synchronize()
        N.call("tg_leaf_stage_open", self.device.handle, arr, len(trees), int(on_device), ctypes.byref(self._h))
        hh, lv = ctypes.c_int(), ctypes.c_int()
        N.call("tg_leaf_stage_height", self._h, ctypes.byref(hh), ctypes.byref(lv))
        self.height = hh.value

    def root(self, k: int):
        t = self.trees[k]
        n = (1 << t.s) if isinstance(t, Forest) else 2
        out = np.zeros(2 * n, dtype=np.uint64)
        N.call("tg_leaf_stage_root", self._h, k, out.ctypes.data)
        return _pairs(out, n)

    def prove_level(self, transcript: Transcript) -> LevelRecord:
        cap = 64
        rootc = np.zeros(2 * cap, dtype=np.uint64)
        rounds = np.zeros(6 * cap, dtype=np.uint64)
        chal = np.zeros(2 * cap, dtype=np.uint64)
        claims = np.zeros(2 * (cap + 1), dtype=np.uint64)
        evals = np.zeros(8 * len(self.trees), dtype=np.uint64)
        present = np.zeros(len(self.trees), dtype=np.int32)
        o = N.TreeLevelProofC()
        o.root_challenges, o.rounds, o.challenges = rootc.ctypes.data, rounds.ctypes.data, chal.ctypes.data
        o.claims, o.evals, o.present = claims.ctypes.data, evals.ctypes.data, present.ctypes.data
        N.call("tg_leaf_stage_prove_level", self._h, ctypes.byref(transcript.raw), ctypes.byref(o))
        n = o.n_max
        return LevelRecord(f"tree/{o.level}", _pairs(rootc, o.n_root_challenges), (int(o.gamma[0]), int(o.gamma[1])),
                           (int(o.lambda_[0]), int(o.lambda_[1])) if o.has_lambda else None,
                           [_pairs(rounds[6 * j:6 * j + 6], 3) for j in range(n)], _pairs(chal, n),
                           _pairs(claims, n + 1), _pairs(evals, o.n_evals), (int(o.rho[0]), int(o.rho[1])),
                           [int(x) for x in present[:o.n_present]], transcript.state, transcript.counter)

    def claim(self, k: int):
        """(point, claim, level): a forest's claim is its value, a fraction tree's (p, q)."""
        pt = np.zeros(2 * 80, dtype=np.uint64)
        npt, own = ctypes.c_int(), ctypes.c_int()
        c = np.zeros(4, dtype=np.uint64)
        N.call("tg_leaf_stage_claim", self._h, k, pt.ctypes.data, ctypes.byref(npt), c.ctypes.data, ctypes.byref(own))
        claim = _pairs(c, 1)[0] if isinstance(self.trees[k], Forest) else tuple(_pairs(c, 2))
        return _pairs(pt, npt.value), claim, own.value

    def prove(self, transcript: Transcript) -> list[LevelRecord]:
        return [self.prove_level(transcript) for _ in range(self.height)]

    def close(self):
        if self._h:
            N.call("tg_leaf_stage_close", self._h)
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def prove_trees(transcript: Transcript, leaves: list, device: Device | None = None) -> list[LevelRecord]:
    """A batch of product trees (each a single tree from its Fp2 leaves), level by level."""
    with LeafStage([Forest(0, lv) for lv in leaves], device) as st:
        return st.prove(transcript)


def prove_forests(transcript: Transcript, forests: list[Forest], device: Device | None = None) -> list[LevelRecord]:
    with LeafStage(forests, device) as st:
        return st.prove(transcript)


def generated_fraction(height: int, key_seed: int, value_seed: int, mult_seed: int | None, alpha, beta,
                       device: Device | None = None, deferred: bool = False) -> Fraction:
    """A fraction tree of 2^height generated leaves on the device (the reference benchmark's LogUp
    inputs): leaf j is (1 or −m_j, α − (k_j + β·v_j)) from the counter generator; numerators of 1
    (no mult_seed) are not stored. deferred: the leaves are generated when a leaf stage opens the
    tree, in the same pass as its two lowest levels (the tensors hold them from then on)."""
    import torch

    d = resolve(device)
    count = 1 << height
    unit = mult_seed is None
    num = None if unit else torch.empty(2 * count, dtype=torch.int64, device=f"cuda:{d.ordinal}")
    den = torch.empty(2 * count, dtype=torch.int64, device=f"cuda:{d.ordinal}")
    if deferred:
        return Fraction(den, num, gen=LeafGen(key_seed, value_seed, mult_seed, tuple(alpha), tuple(beta)))
    torch.cuda.current_stream().synchronize()
    a = (ctypes.c_uint64 * 2)(*alpha)
    b = (ctypes.c_uint64 * 2)(*beta)
    N.call("tg_logup_leaves", d.handle, key_seed, value_seed, int(unit), mult_seed or 0, a, b, count,
           None if unit else num.data_ptr(), den.data_ptr())
    return Fraction(den, num)
