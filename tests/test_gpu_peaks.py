"""The integer-pipe microbenchmarks that give the integer-bound kernels their roofline
denominators: each rate is finite, positive and within physical reach of a GB300."""
import math

import pytest

pytestmark = pytest.mark.gpu


def test_int_peaks():
    from tessera_gb300.device import default_device

    p = default_device().int_peaks()
    assert set(p) == {"imad_wide_per_s", "mulmod_per_s", "butterflies_per_s", "blake3_compressions_per_s"}
    for v in p.values():
        assert math.isfinite(v) and v > 0
    # a product costs several mad.wide, a compression several hundred integer operations
    assert p["mulmod_per_s"] < p["imad_wide_per_s"]
    assert p["blake3_compressions_per_s"] < p["mulmod_per_s"]
    assert p["imad_wide_per_s"] < 1e14
