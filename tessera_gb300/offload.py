"""Tree-level offload on the GPU: the reference's LevelOffload/DeviceLevel seam
(crates/tessera-sumcheck/src/offload.rs:17-79), implemented as its GpuLevels is
(crates/tessera-gpu/src/level.rs:52-146): load() copies an instance's Fp2 tables to the device
or declines, sums() and bind() run each remaining round there, firsts() reads the final
evaluations. Thread-safe, as the seam's Send + Sync requires.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _native as N
from .device import Device, host_u64, ptr, resolve


@dataclass
class LevelShape:
    """Fraction: N0·D1 + N1·D0 + λ·D0·D1 over [N0, N1, D0, D1]; product: V0·V1 over [V0, V1]."""

    kind: str
    lam: tuple[int, int] = (0, 0)

    @classmethod
    def fraction(cls, lam) -> "LevelShape":
        return cls("fraction", (int(lam[0]), int(lam[1])))

    @classmethod
    def product(cls) -> "LevelShape":
        return cls("product")


def _fp2_words(values) -> np.ndarray:
    a = host_u64(values)
    return a.reshape(-1)


class DeviceLevel:
    def __init__(self, handle, ntables: int):
        self._h = handle
        self.ntables = ntables

    def sums(self, low, high, low_bits: int) -> list[tuple[int, int]]:
        lo, hi = _fp2_words(low), _fp2_words(high)
        if lo.size != 2 << low_bits:
            raise ValueError(f"low holds 2^{low_bits} Fp2 values")
        out = (ctypes.c_uint64 * 6)()
        N.call("tg_level_sums", self._h, ptr(lo), ptr(hi), hi.size // 2, low_bits, out)
        return [(int(out[0]), int(out[1])), (int(out[2]), int(out[3])), (int(out[4]), int(out[5]))]

    def bind(self, r):
        rr = (ctypes.c_uint64 * 2)(int(r[0]), int(r[1]))
        N.call("tg_level_bind", self._h, rr)

    def firsts(self) -> list[tuple[int, int]]:
        out = (ctypes.c_uint64 * (2 * self.ntables))()
        N.call("tg_level_firsts", self._h, out)
        return [(int(out[2 * k]), int(out[2 * k + 1])) for k in range(self.ntables)]

    def close(self):
        if self._h:
            N.lib().tg_level_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class GpuLevels:
    """A device that takes level instances up to the device's budget, none below its minimum."""

    def __init__(self, device: Device | None = None):
        self.device = resolve(device)

    def load(self, shape: LevelShape, tables) -> DeviceLevel | None:
        arrs = [_fp2_words(t) for t in tables]
        length = arrs[0].size // 2 if arrs else 0
        ptrs = (ctypes.c_void_p * max(1, len(arrs)))(*[a.ctypes.data for a in arrs])
        lam = (ctypes.c_uint64 * 2)(*shape.lam)
        h = ctypes.c_void_p()
        if any(a.size != 2 * length for a in arrs):
            return None
        rc = N.call("tg_level_load", self.device.handle, 0 if shape.kind == "fraction" else 1, lam, ptrs, len(arrs),
                    length, ctypes.byref(h))
        if rc == N.TG_DECLINED:
            return None
        return DeviceLevel(h, len(arrs))
