"""GPU parity of the standalone transforms (NttPlan::{ntt, intt, coset_ntt, coset_intt},
crates/tessera-pcs/src/ntt.rs:461-516): every NTT case of the reference's encoding vectors in both
directions and on the coset, the oracle's transforms at every size from 2^1 to 2^22 over several
rows, round trips at full size on the device, and the refusals."""
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


def test_ntt_golden_vectors(dev):
    """values = ntt(coefficients), coset_values = coset_ntt(coefficients, 7), and both inverses,
    through the host entry points and, all cases of one size stacked, the device ones."""
    import torch

    from tessera_gb300.pcs import NttPlan

    cases = load("encoding")["ntt"]
    for c in cases:
        n = len(c["coefficients"])
        plan = NttPlan(n.bit_length() - 1, device=dev)
        coeffs = np.array([num(x) for x in c["coefficients"]], dtype=np.uint64)
        values = np.array([num(x) for x in c["values"]], dtype=np.uint64)
        coset = np.array([num(x) for x in c["coset_values"]], dtype=np.uint64)
        assert np.array_equal(plan.ntt(coeffs), values), n
        assert np.array_equal(plan.coset_ntt(coeffs, 7), coset), n
        assert np.array_equal(plan.intt(values), coeffs), n
        assert np.array_equal(plan.coset_intt(coset, 7), coeffs), n
    by_size = {}
    for c in cases:
        by_size.setdefault(len(c["coefficients"]), []).append(c)
    for n, cs in by_size.items():
        plan = NttPlan(n.bit_length() - 1, device=dev)
        rows = np.array([[num(x) for x in c["coefficients"]] for c in cs], dtype=np.uint64)
        t = torch.from_numpy(rows.view(np.int64).copy()).cuda()
        plan.ntt(t)
        assert np.array_equal(t.cpu().numpy().view(np.uint64), np.array([[num(x) for x in c["values"]] for c in cs],
                                                                         dtype=np.uint64)), n
        plan.intt(t)
        assert np.array_equal(t.cpu().numpy().view(np.uint64), rows), n


@pytest.mark.parametrize("log_n", list(range(1, 23)))
def test_ntt_matches_oracle(dev, log_n):
    """Every size the device transforms take, the single-CTA (n ≤ 2^12) and the register-resident
    (2^13..2^22) paths: each kind over several rows equals the oracle's transform row by row."""
    from tessera_gb300.pcs import NttPlan

    rows = 3 if log_n <= 20 else 2
    n = 1 << log_n
    x = O.splitmix(0x4E54 + log_n, rows * n).reshape(rows, n)
    shift = int(O.splitmix(0x5348 + log_n, 1)[0]) or 7
    plan = NttPlan(log_n, device=dev)
    for name, coset, inverse in [("ntt", None, False), ("intt", None, True), ("coset_ntt", shift, False),
                                 ("coset_intt", shift, True)]:
        got = getattr(plan, name)(x, shift) if coset else getattr(plan, name)(x)
        got = got.reshape(rows, n)
        for r in range(rows):
            assert np.array_equal(got[r], O.ntt(x[r], coset=coset, inverse=inverse)), (name, log_n, r)


@pytest.mark.parametrize("log_n,rows", [(20, 64), (22, 16)])
def test_ntt_round_trips_on_device(dev, log_n, rows):
    """intt(ntt(x)) = x and coset_intt(coset_ntt(x, g), g) = x over many rows in device memory,
    and ntt is linear: ntt(x + y) = ntt(x) + ntt(y) (checked on one row against the host)."""
    import torch

    from tessera_gb300.pcs import NttPlan
    from tessera_gb300.workloads import fill_device

    n = 1 << log_n
    plan = NttPlan(log_n, device=dev)
    x = fill_device(torch.empty(rows * n, dtype=torch.int64, device="cuda"), 0x52540 + log_n, dev)
    torch.cuda.synchronize()
    keep = x.clone()
    plan.ntt(x)
    assert not torch.equal(x, keep)
    plan.intt(x)
    torch.cuda.synchronize()
    assert torch.equal(x, keep)
    g = 0x1234567890ABCDEF
    plan.coset_ntt(x, g)
    plan.coset_intt(x, g)
    torch.cuda.synchronize()
    assert torch.equal(x, keep)
    a = keep[:n].cpu().numpy().view(np.uint64)
    b = keep[n:2 * n].cpu().numpy().view(np.uint64)
    s = O.fp_vec("add", a, b)
    fa, fb, fs = plan.ntt(a), plan.ntt(b), plan.ntt(s)
    assert np.array_equal(fs, O.fp_vec("add", fa, fb))


def test_ntt_refusals(dev):
    from tessera_gb300 import _native as N
    from tessera_gb300.pcs import NttPlan

    with pytest.raises(ValueError):
        NttPlan(23, device=dev)
    plan = NttPlan(4, device=dev)
    x = np.arange(16, dtype=np.uint64)
    with pytest.raises(ValueError):
        plan.coset_ntt(x, 0)
    with pytest.raises(ValueError):
        plan.ntt(x[:15])
    with pytest.raises(N.InvalidInput):
        N.call("tg_coset_ntt", dev.handle, 4, P, x.ctypes.data, 1)  # a non-canonical shift
    with pytest.raises(N.InvalidInput):
        N.call("tg_ntt", dev.handle, 23, x.ctypes.data, 1)
    assert np.array_equal(NttPlan(0, device=dev).ntt(np.array([5], dtype=np.uint64)), [5])
