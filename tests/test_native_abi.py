"""CPU checks of the C ABI: the library loads, exports every function include/tessera_gb300.h
declares, and its host-side code (BLAKE3 domain hashing, the Fiat–Shamir transcript) reproduces
the reference's golden vectors. No call here touches a GPU."""
import ctypes
import re
from pathlib import Path

import pytest

from golden_data import blake3_input, load, num
from tessera_gb300 import _native as N
from tessera_gb300.hash import Transcript, hash as tg_hash

HEADER = Path(__file__).resolve().parent.parent / "include" / "tessera_gb300.h"


def declared_functions():
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    return sorted(set(re.findall(r"\b(tg_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(str(N.LIB_PATH))
    names = declared_functions()
    assert len(names) >= 38
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_bindings_cover_the_header():
    assert set(declared_functions()) == set(N.SIGNATURES)


def test_host_domain_hash():
    v = load("hash")
    for d in v["domains"]:
        for n, digest in zip(v["input_lengths"], d["digests"]):
            assert tg_hash(d["name"], blake3_input(n)).hex() == digest


def test_host_transcript_sessions():
    for c in load("transcript")["cases"]:
        t = Transcript(bytes.fromhex(c["context_tce"]))
        assert t.state.hex() == c["state"]
        for s in c["steps"]:
            op = s["op"]
            if op == "absorb":
                t.absorb(s["label"], bytes.fromhex(s["tce"]))
            elif op == "squeeze":
                assert t.squeeze(s["label"]).hex() == s["out"]
            elif op == "challenge_fp2":
                assert list(t.challenge_fp2(s["label"])) == [num(x) for x in s["value"]]
            elif op == "challenge_fp":
                assert t.challenge_fp(s["label"]) == num(s["value"])
            elif op == "challenge_indices":
                assert t.challenge_indices(s["label"], s["log_n"], s["count"]) == [num(x) for x in s["value"]]
            elif op == "grind":
                # the GPU search is tested on the GPU; here the host check replays the nonce
                assert t.check_grind(s["label"], s["bits"], num(s["nonce"]))
            elif op == "check_grind":
                assert t.check_grind(s["label"], s["bits"], num(s["nonce"])) == s["valid"]
            assert t.state.hex() == s["state"] and t.counter == s["counter"]


def test_transcript_refuses_non_printable_label():
    t = Transcript(bytes(10))
    with pytest.raises(N.InvalidInput):
        t.absorb("bad\nlabel", b"")


def test_device_calls_fail_loudly_without_a_gpu():
    try:
        import torch

        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    h = ctypes.c_void_p()
    with pytest.raises(N.TesseraError):
        N.call("tg_device_open", 0, None, ctypes.byref(h))


def test_host_prefault():
    """tg_host_prefault reads every page of a host buffer and touches nothing on a device."""
    import numpy as np

    buf = np.arange(3 << 17, dtype=np.uint64)
    before = buf.copy()
    N.call("tg_host_prefault", ctypes.c_void_p(buf.ctypes.data), buf.nbytes)
    N.call("tg_host_prefault", ctypes.c_void_p(buf.ctypes.data), 1)
    N.call("tg_host_prefault", None, 0)
    assert np.array_equal(buf, before)
    with pytest.raises(N.TesseraError):
        N.call("tg_host_prefault", None, 8)
