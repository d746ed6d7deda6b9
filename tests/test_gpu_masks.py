"""GPU parity of the advice mask stream (ProverDomain::AdviceMasks, crates/tessera-hash/src/
domain.rs:83-127): the vectors' 24 masks of their proof seed and the pinned seed whose word 6 is
rejected, and the oracle's stream at a million values from an offset, through the host and the
device entry points."""
import numpy as np
import pytest

from golden_data import load, num
from oracle import oracle as O

pytestmark = pytest.mark.gpu
P = 0xFFFFFFFF00000001


@pytest.fixture(scope="module")
def dev():
    from tessera_gb300.device import default_device

    return default_device()


def oracle_values(seed: bytes, words: int):
    raw = O.blake3("derive", seed, 8 * words, key="tessera/v1/advice-masks")
    w = np.frombuffer(raw, dtype="<u8")
    return w[w < np.uint64(P)]


def test_advice_masks_golden(dev):
    from tessera_gb300.hash import advice_masks

    ps = load("hash")["prover_streams"]
    got = advice_masks(bytes.fromhex(ps["proof_seed"]), 24, device=dev)
    assert [int(x) for x in got] == [num(x) for x in ps["advice_masks"]]
    rj = ps["rejection"]
    got = advice_masks(bytes.fromhex(rj["seed"]), 15, device=dev)
    assert [int(x) for x in got] == [num(x) for x in rj["values"]]
    # a window across the rejected word
    got = advice_masks(bytes.fromhex(rj["seed"]), 4, first=4, device=dev)
    assert [int(x) for x in got] == [num(x) for x in rj["values"][4:8]]


@pytest.mark.parametrize("first,count", [(0, 1), (12345, 1 << 20), (7, 1000)])
def test_advice_masks_match_oracle(dev, first, count):
    import ctypes

    import torch

    from tessera_gb300 import _native as N
    from tessera_gb300.device import torch_stream
    from tessera_gb300.hash import advice_masks

    seed = bytes(range(32))
    want = oracle_values(seed, first + count + 64)[first:first + count]
    assert len(want) == count
    got = advice_masks(seed, count, first=first, device=dev)
    assert np.array_equal(got, want)
    out = torch.full((count,), -1, dtype=torch.int64, device="cuda")
    buf = ctypes.create_string_buffer(seed, 32)
    N.call("tg_advice_masks_dev", dev.handle, buf, 32, first, count, ctypes.c_void_p(out.data_ptr()), torch_stream())
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy().view(np.uint64), want)


def test_advice_masks_refusals(dev):
    from tessera_gb300 import _native as N
    from tessera_gb300.hash import advice_masks

    with pytest.raises(N.InvalidInput):
        advice_masks(bytes(65), 4, device=dev)  # a seed longer than one BLAKE3 block
    assert len(advice_masks(bytes(32), 0, device=dev)) == 0
