"""One GPU, opened once: the handle every call of the package runs on.

Mirrors the reference's backend selection (crates/tessera-prover/src/gpu.rs:111-146: one
device, budgets from TESSERA_GPU_LEVEL_GIB / TESSERA_GPU_LEVEL_MIN).
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

from . import _native as N

P = 0xFFFFFFFF00000001


class Device:
    """An open GPU. `level_budget_bytes` and `level_min_entries` bound the level offload;
    `lde_group_bytes` sizes the encoder's L2-resident scratch per group of rows; `tree_sum_q1`
    makes every tree-level round sum q(1) instead of deriving it from its claim (same proofs; a
    check of that path)."""

    def __init__(self, ordinal: int = 0, level_budget_bytes: int | None = None, level_min_entries: int | None = None,
                 lde_group_bytes: int = 0, tree_sum_q1: bool = False):
        if level_budget_bytes is None:
            gib = os.environ.get("TESSERA_GPU_LEVEL_GIB")
            level_budget_bytes = int(float(gib) * (1 << 30)) if gib else 0
        if level_min_entries is None:
            level_min_entries = int(os.environ.get("TESSERA_GPU_LEVEL_MIN", "0"))
        cfg = N.Config(level_budget_bytes, level_min_entries, lde_group_bytes, N.TG_TREE_SUM_Q1 if tree_sum_q1 else 0)
        h = ctypes.c_void_p()
        N.call("tg_device_open", ordinal, ctypes.byref(cfg), ctypes.byref(h))
        self.handle = h
        self.ordinal = ordinal

    def close(self):
        if self.handle:
            N.lib().tg_device_close(self.handle)
            self.handle = None

    def trim(self):
        """Returns the workspace memory closed leaf stages left for reuse to the driver."""
        N.call("tg_device_trim", self.handle)

    def sync(self):
        N.call("tg_device_sync", self.handle)

    def stream_ptr(self) -> int:
        """The handle's CUDA stream (where calls without an explicit stream run)."""
        s = ctypes.c_void_p()
        N.call("tg_device_stream", self.handle, ctypes.byref(s))
        return s.value or 0

    def launches(self) -> int:
        n = ctypes.c_uint64()
        N.call("tg_device_launches", self.handle, ctypes.byref(n))
        return n.value

    def int_peaks(self) -> dict:
        """Measured integer-pipe rates of this GPU (per second): mad.wide.u32, Goldilocks
        products, radix-2 butterflies in radix-32 shift-twiddle transforms, BLAKE3 compressions."""

        class _Peaks(ctypes.Structure):
            _fields_ = [("imad_wide_per_s", ctypes.c_double), ("mulmod_per_s", ctypes.c_double),
                        ("butterflies_per_s", ctypes.c_double), ("blake3_compressions_per_s", ctypes.c_double)]

        p = _Peaks()
        N.call("tg_measure_int_peaks", self.handle, ctypes.byref(p))
        return {name: getattr(p, name) for name, _ in _Peaks._fields_}

    def check_lazy_arith(self, words):
        """The device's lazy field arithmetic on any 64-bit words (tg_check_lazy_arith): an array
        of shape (n, 16) of canonical results, in the order the header lists."""
        import numpy as np

        w = np.ascontiguousarray(np.asarray(words, dtype=np.uint64))
        out = np.zeros((len(w), 16), dtype=np.uint64)
        N.call("tg_check_lazy_arith", self.handle, ctypes.c_void_p(w.ctypes.data), len(w),
               ctypes.c_void_p(out.ctypes.data))
        return out

    def profile(self, on: bool = True):
        N.call("tg_profile_enable", self.handle, int(on))

    def profile_read(self) -> dict:
        """{kernel: (ms, launches, units)} since the last read."""
        cap = 64
        names = ctypes.create_string_buffer(8192)
        ms = (ctypes.c_double * cap)()
        cnt = (ctypes.c_uint64 * cap)()
        units = (ctypes.c_uint64 * cap)()
        count = ctypes.c_size_t()
        N.call("tg_profile_read", self.handle, names, 8192, ms, cnt, units, cap, ctypes.byref(count))
        keys = [k for k in names.value.decode().split("\n") if k]
        return {k: (ms[i], int(cnt[i]), int(units[i])) for i, k in enumerate(keys[:cap])}

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default = None
_default_lock = threading.Lock()


def default_device() -> Device:
    """The process's device 0, opened on first use."""
    global _default
    with _default_lock:
        if _default is None:
            _default = Device(0)
        return _default


def resolve(device: Device | None) -> Device:
    return device if device is not None else default_device()


# ---- buffers ----------------------------------------------------------------------------------

def host_u64(x) -> np.ndarray:
    """A C-contiguous uint64 view or copy of `x` (field words)."""
    a = np.ascontiguousarray(np.asarray(x, dtype=np.uint64))
    return a


def ptr(a: np.ndarray):
    return ctypes.c_void_p(a.ctypes.data) if a is not None and a.size else None


def is_device_tensor(x) -> bool:
    return hasattr(x, "is_cuda") and bool(getattr(x, "is_cuda"))


def dev_ptr(x) -> ctypes.c_void_p:
    """The device address of a CUDA tensor (int64/uint64/uint8 storage used as raw words)."""
    if not is_device_tensor(x):
        raise TypeError("expected a CUDA tensor")
    if not x.is_contiguous():
        raise ValueError("device buffers must be contiguous")
    return ctypes.c_void_p(x.data_ptr())


def torch_stream() -> ctypes.c_void_p:
    """torch's current CUDA stream, so library work on torch-owned buffers stays in order."""
    import torch

    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def digests(buf: np.ndarray) -> list[bytes]:
    b = np.ascontiguousarray(buf, dtype=np.uint8).reshape(-1, 32)
    return [bytes(r) for r in b]
