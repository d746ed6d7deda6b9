"""tessera_gb300: the Tessera proving hot path, GB300-native.

Goldilocks NTT/LDE, BLAKE3 column chains and Merkle roots, batched sumcheck and tree-level
offload, as hand-written sm_103a kernels behind a C ABI (include/tessera_gb300.h, built into
tessera_gb300/_build/libtessera_gb300.so). The Python modules mirror the reference's crate
interfaces (tessera-hash, tessera-pcs, tessera-sumcheck) so that the device path is a drop-in.
There is no CPU fallback: without the built library every entry point raises.
"""
from . import _native
from .device import Device, default_device

__all__ = ["Device", "default_device", "_native"]


def library_path():
    return _native.LIB_PATH
