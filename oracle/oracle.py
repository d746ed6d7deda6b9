"""TEST INFRASTRUCTURE ONLY: ctypes bindings of the CPU oracle (``tessera_oracle.c``).

The oracle restates the reference's Rust algorithms in plain C. The test suite uses it as the
checker of the CUDA path, ``__graft_entry__.smoke`` checks one small case against it, and
``bench.py`` times it as the CPU baseline. The product package never imports this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "libtessera_oracle.so"

P = 0xFFFFFFFF00000001

_lib = None


def build() -> Path:
    """Compiles the oracle with its Makefile (gcc, a few seconds)."""
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB_PATH


def build_baseline() -> None:
    """The GPU baseline: the reference's own kernels compiled from its checkout (when present)
    into oracle/_ref/, and the harness that drives them, oracle/_build/librefgpu.so."""
    subprocess.run(["make", "-s", "-C", str(HERE), "ref", "refgpu"], check=True)


def lib():
    global _lib
    if _lib is None:
        src = HERE / "tessera_oracle.c"
        if not LIB_PATH.exists() or LIB_PATH.stat().st_mtime < src.stat().st_mtime:
            build()
        _lib = ctypes.CDLL(str(LIB_PATH))
        _declare(_lib)
    return _lib


u64p = ctypes.POINTER(ctypes.c_uint64)
u8p = ctypes.POINTER(ctypes.c_uint8)


class Table(ctypes.Structure):
    _fields_ = [("values", u64p), ("is_ext", ctypes.c_int), ("is_public", ctypes.c_int)]


class Instance(ctypes.Structure):
    _fields_ = [("tables", ctypes.POINTER(Table)), ("ntables", ctypes.c_int), ("vars", ctypes.c_int)]


class Transcript(ctypes.Structure):
    _fields_ = [("state", ctypes.c_uint8 * 32), ("counter", ctypes.c_uint64)]


def _declare(L):
    U64, SZ, INT, U32 = ctypes.c_uint64, ctypes.c_size_t, ctypes.c_int, ctypes.c_uint32
    vp = ctypes.c_void_p
    sig = {
        "or_fp_add": (U64, [U64, U64]),
        "or_fp_sub": (U64, [U64, U64]),
        "or_fp_mul": (U64, [U64, U64]),
        "or_fp_pow": (U64, [U64, U64]),
        "or_fp_inv": (U64, [U64]),
        "or_fp_reduce": (U64, [U64]),
        "or_root_of_unity": (U64, [U32]),
        "or_fp2_mul": (None, [vp, vp, vp]),
        "or_fp2_inv": (None, [vp, vp]),
        "or_fp_vec": (None, [INT, vp, vp, vp, SZ]),
        "or_fp2_vec_mul": (None, [vp, vp, vp, SZ]),
        "or_blake3": (None, [INT, vp, vp, SZ, vp, SZ]),
        "or_context_key": (None, [ctypes.c_char_p, vp]),
        "or_hash": (None, [ctypes.c_char_p, vp, SZ, vp]),
        "or_column_init": (None, [vp, U64, vp, INT]),
        "or_column_absorb": (None, [vp, U64, vp, SZ, INT]),
        "or_merkle_tree": (None, [vp, SZ, vp, INT]),
        "or_merkle_root": (None, [vp, SZ, vp, INT]),
        "or_merkle_node": (None, [vp, vp, vp]),
        "or_transcript_init": (None, [vp, vp, SZ]),
        "or_transcript_absorb": (None, [vp, ctypes.c_char_p, vp, SZ]),
        "or_transcript_squeeze": (None, [vp, ctypes.c_char_p, vp]),
        "or_transcript_challenge_fp2": (None, [vp, ctypes.c_char_p, vp]),
        "or_transcript_absorb_fp2s": (None, [vp, ctypes.c_char_p, vp, SZ]),
        "or_transcript_challenge_fp": (U64, [vp, ctypes.c_char_p]),
        "or_transcript_challenge_indices": (None, [vp, ctypes.c_char_p, U32, U32, vp]),
        "or_transcript_pow_meets": (INT, [vp, ctypes.c_char_p, U32, U64]),
        "or_transcript_grind": (U64, [vp, ctypes.c_char_p, U32]),
        "or_ntt": (None, [vp, U32]),
        "or_intt": (None, [vp, U32]),
        "or_coset_ntt": (None, [vp, U32, U64]),
        "or_coset_intt": (None, [vp, U32, U64]),
        "or_encode_rows": (INT, [U32, U32, U32, vp, SZ, vp, vp, INT]),
        "or_commit_unmasked": (INT, [U32, U32, U32, vp, vp, SZ, vp, vp, vp, INT]),
        "or_segment_chains": (None, [vp, U64, U32, vp, SZ, vp, INT]),
        "or_merge_segments": (None, [vp, SZ, U64, vp, vp]),
        "or_prove_batch": (INT, [vp, ctypes.c_char_p, INT, vp, INT, vp, vp, vp, vp, ctypes.POINTER(SZ)]),
        "or_level_sums": (None, [INT, vp, vp, SZ, vp, vp, U32, vp]),
        "or_level_bind": (None, [vp, INT, SZ, vp]),
        "or_splitmix_fill": (None, [U64, vp, SZ]),
        "or_mle": (None, [vp, INT, U32, vp, vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def u64(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.uint64))


# ---- field ------------------------------------------------------------------------------------

def fp_vec(op: str, a, b) -> np.ndarray:
    a, b = u64(a), u64(b)
    out = np.empty_like(a)
    lib().or_fp_vec({"add": 0, "sub": 1, "mul": 2}[op], _ptr(a), _ptr(b), _ptr(out), a.size)
    return out


def fp2_vec_mul(a, b) -> np.ndarray:
    a, b = u64(a), u64(b)
    out = np.empty_like(a)
    lib().or_fp2_vec_mul(_ptr(a), _ptr(b), _ptr(out), a.size // 2)
    return out


def splitmix(seed: int, n: int) -> np.ndarray:
    out = np.empty(n, dtype=np.uint64)
    lib().or_splitmix_fill(seed, _ptr(out), n)
    return out


# ---- hashing ----------------------------------------------------------------------------------

def blake3(mode: str, data: bytes, out_len: int = 32, key=None) -> bytes:
    out = ctypes.create_string_buffer(out_len)
    buf = ctypes.create_string_buffer(bytes(data), len(data) or 1)
    if mode == "hash":
        lib().or_blake3(0, None, buf, len(data), out, out_len)
    elif mode == "keyed":
        k = ctypes.create_string_buffer(bytes(key), 32)
        lib().or_blake3(1, k, buf, len(data), out, out_len)
    else:
        k = ctypes.create_string_buffer(key.encode())
        lib().or_blake3(2, k, buf, len(data), out, out_len)
    return out.raw[:out_len]


def hash_domain(name: str, data: bytes) -> bytes:
    out = ctypes.create_string_buffer(32)
    buf = ctypes.create_string_buffer(bytes(data), len(data) or 1)
    lib().or_hash(name.encode(), buf, len(data), out)
    return out.raw


def context_key(name: str) -> bytes:
    out = ctypes.create_string_buffer(32)
    lib().or_context_key(name.encode(), out)
    return out.raw


def column_chains(commitment_id: bytes, rows: np.ndarray, ncols: int, block: int, threads: int = 1) -> np.ndarray:
    """Chains of `ncols` columns over row-major `rows` (m x ncols), in blocks of `block` rows."""
    rows = u64(rows).reshape(-1)
    m = rows.size // ncols if ncols else 0
    chains = np.zeros((ncols, 32), dtype=np.uint8)
    cid = np.frombuffer(bytes(commitment_id), dtype=np.uint8).copy()
    lib().or_segment_chains(_ptr(cid), ncols, block, _ptr(rows), m, _ptr(chains), threads)
    return chains


def merkle_tree(leaves: np.ndarray, threads: int = 1) -> np.ndarray:
    leaves = np.ascontiguousarray(leaves, dtype=np.uint8).reshape(-1, 32)
    n = leaves.shape[0]
    nodes = np.zeros((2 * n - 1, 32), dtype=np.uint8)
    lib().or_merkle_tree(_ptr(leaves), n, _ptr(nodes), threads)
    return nodes


def merkle_root(leaves: np.ndarray, threads: int = 1) -> bytes:
    leaves = np.ascontiguousarray(leaves, dtype=np.uint8).reshape(-1, 32)
    out = ctypes.create_string_buffer(32)
    lib().or_merkle_root(_ptr(leaves), leaves.shape[0], out, threads)
    return out.raw


class OracleTranscript:
    """The reference transcript (tessera-hash/src/transcript.rs), over the oracle's BLAKE3."""

    def __init__(self, context_tce: bytes):
        self.t = Transcript()
        buf = ctypes.create_string_buffer(bytes(context_tce), len(context_tce))
        lib().or_transcript_init(ctypes.byref(self.t), buf, len(context_tce))

    @property
    def state(self) -> bytes:
        return bytes(self.t.state)

    @property
    def counter(self) -> int:
        return int(self.t.counter)

    def absorb(self, label: str, value: bytes):
        buf = ctypes.create_string_buffer(bytes(value), len(value) or 1)
        lib().or_transcript_absorb(ctypes.byref(self.t), label.encode(), buf, len(value))

    def squeeze(self, label: str) -> bytes:
        out = ctypes.create_string_buffer(32)
        lib().or_transcript_squeeze(ctypes.byref(self.t), label.encode(), out)
        return out.raw

    def challenge_fp2(self, label: str):
        out = (ctypes.c_uint64 * 2)()
        lib().or_transcript_challenge_fp2(ctypes.byref(self.t), label.encode(), out)
        return (int(out[0]), int(out[1]))

    def challenge_fp(self, label: str) -> int:
        return int(lib().or_transcript_challenge_fp(ctypes.byref(self.t), label.encode()))

    def challenge_indices(self, label: str, log_n: int, count: int):
        out = np.zeros(max(1, count), dtype=np.uint64)
        lib().or_transcript_challenge_indices(ctypes.byref(self.t), label.encode(), log_n, count, _ptr(out))
        return [int(x) for x in out[:count]]

    def grind(self, label: str, bits: int) -> int:
        return int(lib().or_transcript_grind(ctypes.byref(self.t), label.encode(), bits))

    def check_grind(self, label: str, bits: int, nonce: int) -> bool:
        ok = bool(lib().or_transcript_pow_meets(ctypes.byref(self.t), label.encode(), bits, nonce))
        if ok:
            self.absorb(label, int(nonce).to_bytes(8, "little"))
        return ok


# ---- NTT and encoding -------------------------------------------------------------------------

def ntt(values, coset=None, inverse=False) -> np.ndarray:
    v = u64(values).copy()
    log_n = int(v.size).bit_length() - 1
    L = lib()
    if coset is None:
        (L.or_intt if inverse else L.or_ntt)(_ptr(v), log_n)
    else:
        (L.or_coset_intt if inverse else L.or_coset_ntt)(_ptr(v), log_n, coset)
    return v


def encode_rows(rows, log_k: int, log_inv_rate: int, masks=None, mask_coeffs: int = 0, threads: int = 1) -> np.ndarray:
    rows = u64(rows).reshape(-1)
    k = 1 << log_k
    nrows = rows.size // k
    out = np.zeros(nrows << (log_k + log_inv_rate), dtype=np.uint64)
    m = u64(masks).reshape(-1) if mask_coeffs else None
    rc = lib().or_encode_rows(log_k, log_inv_rate, mask_coeffs, _ptr(rows), nrows, _ptr(m), _ptr(out), threads)
    if rc != 0:
        raise ValueError(f"encode_rows refused: {rc}")
    return out.reshape(nrows, -1)


def commit_unmasked(rows, log_k: int, log_inv_rate: int, row_block: int, commitment_id: bytes,
                    threads: int = 1, keep_codewords: bool = True):
    rows = u64(rows).reshape(-1)
    npolys = rows.size >> log_k
    n = 1 << (log_k + log_inv_rate)
    cw = np.zeros((npolys, n), dtype=np.uint64) if keep_codewords else None
    leaves = np.zeros((n, 32), dtype=np.uint8)
    root = ctypes.create_string_buffer(32)
    cid = np.frombuffer(bytes(commitment_id), dtype=np.uint8).copy()
    rc = lib().or_commit_unmasked(log_k, log_inv_rate, row_block, _ptr(cid), _ptr(rows), npolys,
                                  _ptr(cw), _ptr(leaves), root, threads)
    if rc != 0:
        raise ValueError(f"commit_unmasked refused: {rc}")
    return cw, leaves, root.raw


def merge_segments(segment_chains: np.ndarray):
    seg = np.ascontiguousarray(segment_chains, dtype=np.uint8)
    S, n = seg.shape[0], seg.shape[1]
    leaves = np.zeros((n, 32), dtype=np.uint8)
    root = ctypes.create_string_buffer(32)
    lib().or_merge_segments(_ptr(seg), S, n, _ptr(leaves), root)
    return leaves, root.raw


# ---- sumcheck ---------------------------------------------------------------------------------

def prove_batch(transcript: OracleTranscript, prefix: str, degree: int, instances):
    """instances: list of lists of (values: np.uint64 array, is_ext, is_public); an ext table's
    array holds interleaved (c0, c1) words. Returns (gamma, rounds[n_max][degree], challenges,
    final_evals) as tuples of ints."""
    keep = []
    inst_arr = (Instance * len(instances))()
    n_max = 0
    for i, tables in enumerate(instances):
        tarr = (Table * len(tables))()
        vars_ = None
        for k, (vals, is_ext, is_public) in enumerate(tables):
            a = u64(vals)
            keep.append(a)
            tarr[k].values = a.ctypes.data_as(u64p)
            tarr[k].is_ext = int(is_ext)
            tarr[k].is_public = int(is_public)
            length = a.size // (2 if is_ext else 1)
            vars_ = length.bit_length() - 1
        keep.append(tarr)
        inst_arr[i].tables = tarr
        inst_arr[i].ntables = len(tables)
        inst_arr[i].vars = vars_
        n_max = max(n_max, vars_)
    n_evals_cap = sum(len(t) for t in instances)
    gamma = np.zeros(2, dtype=np.uint64)
    rounds = np.zeros(max(1, n_max) * degree * 2, dtype=np.uint64)
    chal = np.zeros(max(1, n_max) * 2, dtype=np.uint64)
    evals = np.zeros(max(1, n_evals_cap) * 2, dtype=np.uint64)
    ne = ctypes.c_size_t(0)
    rc = lib().or_prove_batch(ctypes.byref(transcript.t), prefix.encode(), degree, inst_arr, len(instances),
                              _ptr(gamma), _ptr(rounds), _ptr(chal), _ptr(evals), ctypes.byref(ne))
    if rc != 0:
        raise ValueError(f"prove_batch refused: {rc}")
    pairs = lambda a, n: [(int(a[2 * i]), int(a[2 * i + 1])) for i in range(n)]
    rr = [pairs(rounds[j * degree * 2:(j + 1) * degree * 2], degree) for j in range(n_max)]
    return (int(gamma[0]), int(gamma[1])), rr, pairs(chal, n_max), pairs(evals, ne.value)


def level_sums(shape: str, lam, tables, low, high, low_bits: int):
    tabs = [u64(t) for t in tables]
    ptrs = (ctypes.c_void_p * len(tabs))(*[t.ctypes.data for t in tabs])
    lam_a = u64(lam if lam is not None else (0, 0))
    low, high = u64(low), u64(high)
    out = np.zeros(6, dtype=np.uint64)
    lib().or_level_sums(0 if shape == "fraction" else 1, _ptr(lam_a), ptrs, tabs[0].size // 2, _ptr(low), _ptr(high),
                        low_bits, _ptr(out))
    return [(int(out[0]), int(out[1])), (int(out[2]), int(out[3])), (int(out[4]), int(out[5]))]


def level_bind(tables, r):
    tabs = [u64(t).copy() for t in tables]
    ptrs = (ctypes.c_void_p * len(tabs))(*[t.ctypes.data for t in tabs])
    ra = u64(r)
    lib().or_level_bind(ptrs, len(tabs), tabs[0].size // 2, _ptr(ra))
    return [t[: t.size // 2] for t in tabs]


def mle(values, point, is_ext: bool = False):
    """Σ_x values[x]·eq(point, x), point a list of Fp2 pairs (x_1 the index's lowest bit)."""
    v = u64(values).reshape(-1)
    pt = np.array([c for p_ in point for c in p_], dtype=np.uint64) if point else np.zeros(1, dtype=np.uint64)
    out = (ctypes.c_uint64 * 2)()
    lib().or_mle(_ptr(v), int(is_ext), len(point), _ptr(pt), out)
    return (int(out[0]), int(out[1]))


def threads_available() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1
