"""The allocation-free encoder, tg_encode_rows_noalloc_dev, called through the C ABI.

It is for callers that cannot call cudaMalloc (device memory owned by another allocator, or a
loop that must not synchronize the device the way cudaMalloc and cudaFree do): its tables and
scratch live in a fixed 32 MiB device array instead. Its codewords must equal those of the
allocating entry point, tg_encode_rows_dev, bit for bit, on consecutive calls that reuse and then
replace the array's contents, and a call must leave the device's free memory unchanged.

This file is collected last, so a run that stops at its first failure has run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _encode(fn, dev, log_k, log_r, P, rows_d, nrows, masks_d, out_d):
    from tessera_gb300 import _native as N
    from tessera_gb300.device import torch_stream

    rc = getattr(N.lib(), fn)(dev.handle, log_k, log_r, P, ctypes.c_void_p(rows_d.data_ptr()), nrows,
                              ctypes.c_void_p(masks_d.data_ptr()) if masks_d is not None else None,
                              ctypes.c_void_p(out_d.data_ptr()), torch_stream())
    N.check(rc)


@pytest.mark.parametrize("calls", [[(14, 1, 5, 3), (14, 1, 0, 2)], [(16, 2, 0, 2), (8, 3, 7, 5)], [(19, 1, 3, 1), (12, 1, 4096, 4)]])
def test_noalloc_matches_allocating_encoder(calls):
    import torch

    from tessera_gb300.device import default_device

    dev = default_device()
    for i, (log_k, log_r, P, nrows) in enumerate(calls):
        k, n = 1 << log_k, 1 << (log_k + log_r)
        rng = np.random.default_rng(1000 * log_k + 10 * log_r + i)
        rows = rng.integers(0, 0xFFFFFFFF00000001, size=nrows * k, dtype=np.uint64)
        masks = rng.integers(0, 0xFFFFFFFF00000001, size=max(1, nrows * P), dtype=np.uint64)
        rows_d = torch.from_numpy(rows.view(np.int64)).cuda()
        masks_d = torch.from_numpy(masks.view(np.int64)).cuda() if P else None
        want = torch.empty(nrows * n, dtype=torch.int64, device="cuda")
        got = torch.full((nrows * n,), -1, dtype=torch.int64, device="cuda")
        _encode("tg_encode_rows_dev", dev, log_k, log_r, P, rows_d, nrows, masks_d, want)
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        _encode("tg_encode_rows_noalloc_dev", dev, log_k, log_r, P, rows_d, nrows, masks_d, got)
        torch.cuda.synchronize()
        free1 = torch.cuda.mem_get_info()[0]
        assert torch.equal(got, want), (log_k, log_r, P, nrows)
        if i > 0:  # the first call may load the library's module, which places the fixed array
            assert free1 == free0, "the allocation-free encoder changed the device's free memory"


def test_noalloc_refuses_shapes_beyond_its_array():
    import torch

    from tessera_gb300 import _native as N
    from tessera_gb300.device import default_device

    dev = default_device()
    rows_d = torch.zeros(1 << 20, dtype=torch.int64, device="cuda")
    out_d = torch.zeros(1 << 21, dtype=torch.int64, device="cuda")
    with pytest.raises(N.InvalidInput, match="fixed scratch"):
        _encode("tg_encode_rows_noalloc_dev", dev, 20, 1, 0, rows_d, 1, None, out_d)


def test_noalloc_graph_replay_after_a_call_of_another_shape():
    """A call recorded into a CUDA graph writes its own tables when the graph runs.

    The fixed array keeps the tables of the last shape encoded. A graph recorded from a call of
    shape A and replayed after a direct call of shape B must still give A's codewords.
    """
    import torch

    from tessera_gb300.device import default_device

    dev = default_device()
    shapes = {"a": (14, 1, 0, 2), "b": (13, 2, 0, 3)}
    bufs = {}
    for name, (log_k, log_r, P, nrows) in shapes.items():
        k, n = 1 << log_k, 1 << (log_k + log_r)
        rng = np.random.default_rng(77 + log_k)
        rows = rng.integers(0, 0xFFFFFFFF00000001, size=nrows * k, dtype=np.uint64)
        rows_d = torch.from_numpy(rows.view(np.int64)).cuda()
        want = torch.empty(nrows * n, dtype=torch.int64, device="cuda")
        _encode("tg_encode_rows_dev", dev, log_k, log_r, P, rows_d, nrows, None, want)
        bufs[name] = (rows_d, want, torch.full((nrows * n,), -1, dtype=torch.int64, device="cuda"))
    torch.cuda.synchronize()
    a, b = shapes["a"], shapes["b"]
    _encode("tg_encode_rows_noalloc_dev", dev, a[0], a[1], a[2], bufs["a"][0], a[3], None, bufs["a"][2])
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream()
    with torch.cuda.graph(graph, stream=side, capture_error_mode="relaxed"):
        _encode("tg_encode_rows_noalloc_dev", dev, a[0], a[1], a[2], bufs["a"][0], a[3], None, bufs["a"][2])
    bufs["a"][2].fill_(-1)
    torch.cuda.synchronize()
    # the direct call runs on the library's stream (torch's default stream has no handle), so the
    # replay waits for it to end: calls that overlap on the GPU race on the array
    _encode("tg_encode_rows_noalloc_dev", dev, b[0], b[1], b[2], bufs["b"][0], b[3], None, bufs["b"][2])
    torch.cuda.synchronize()
    graph.replay()
    torch.cuda.synchronize()
    assert torch.equal(bufs["b"][2], bufs["b"][1])
    assert torch.equal(bufs["a"][2], bufs["a"][1])
    # a direct call of shape A after the replay
    bufs["a"][2].fill_(-1)
    _encode("tg_encode_rows_noalloc_dev", dev, a[0], a[1], a[2], bufs["a"][0], a[3], None, bufs["a"][2])
    torch.cuda.synchronize()
    assert torch.equal(bufs["a"][2], bufs["a"][1])
