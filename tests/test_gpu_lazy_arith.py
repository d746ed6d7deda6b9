"""The device's lazy Goldilocks arithmetic (tg_check_lazy_arith) against exact integer arithmetic.

The hot kernels keep field values as any 64-bit word (x and x − p both stand for x mod p) and sum
products unreduced in five 32-bit limbs; random inputs almost never reach the edges where a carry or
a borrow crosses a limb, so the words here are those edges — 0, p − 1, p, p + 1, 2^32 ± 1, 2^63,
2^64 − 2^32, 2^64 − 1 — in every ordered pair, then words just above p and random words."""
import numpy as np
import pytest

P = (1 << 64) - (1 << 32) + 1
EDGES = [0, 1, 2, 7, P - 2, P - 1, P, P + 1, (1 << 32) - 1, 1 << 32, (1 << 32) + 1, (1 << 63) - 1, 1 << 63,
         (1 << 64) - (1 << 32), (1 << 64) - 2, (1 << 64) - 1, 0xFFFFFFFF00000000 - 1, 0x00000000FFFFFFFE]


@pytest.fixture(scope="module")
def dev():
    from tessera_gb300.device import default_device

    return default_device()


def _words(seed: int) -> list[int]:
    rng = np.random.default_rng(seed)
    w = [x for e1 in EDGES for e2 in EDGES for x in (e1, e2)]
    w += [P + int(r) for r in rng.integers(0, (1 << 32) - 1, size=256, dtype=np.uint64)]
    w += [int(r) for r in rng.integers(0, 1 << 63, size=256, dtype=np.uint64) * 2 + rng.integers(0, 2, size=256, dtype=np.uint64)]
    return w


def _mul2(x0, x1, y0, y1):
    return (x0 * y0 + 7 * x1 * y1) % P, (x0 * y1 + x1 * y0) % P


def _expected(w: list[int]) -> np.ndarray:
    n = len(w)
    rows = []
    for i in range(n):
        a, b, c, d = w[i], w[(i + 1) % n], w[(i + 2) % n], w[(i + 3) % n]
        row = [(a + b) % P, (a - b) % P, a * b % P, 7 * a % P, (a << 5) % P, (a << 40) % P, (a << 70) % P,
               (a * b + c * d) % P, (a + b * c + d * a) % P]
        row += list(_mul2(a, b, c, d))
        f = _mul2(c, d, b, a)
        row += [(a + f[0]) % P, (b + f[1]) % P]
        g1, g2 = _mul2(a, b, c, d), _mul2(b, d, a, c)
        row += [(g1[0] + g2[0]) % P, (g1[1] + g2[1]) % P]
        row.append(sum(w[(i + k) % n] * w[(i + 2 * k + 1) % n] for k in range(64)) % P)
        rows.append(row)
    return np.array(rows, dtype=np.uint64)


@pytest.mark.gpu
@pytest.mark.parametrize("seed", [1, 2])
def test_lazy_arith_matches_integers(dev, seed):
    w = _words(seed)
    got = dev.check_lazy_arith(np.array(w, dtype=np.uint64))
    want = _expected(w)
    bad = np.argwhere(got != want)
    assert bad.size == 0, f"{len(bad)} mismatches, first (word, output) {bad[0].tolist()}"


def test_expected_values_are_canonical():
    """The integer model of the check itself: every expected value is below p, and the edge words
    include values at and above p (lazy words the kernels carry)."""
    w = _words(3)
    e = _expected(w[:64])
    assert (e < np.uint64(P)).all()
    assert any(x >= P for x in w)
