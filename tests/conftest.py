"""Test configuration: the `gpu` marker and shared paths.

Tests marked `gpu` need a CUDA device and the built extension; every other test runs on CPU.
"""
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
for p in (ROOT, ROOT / "tests"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and the built sm_103a library")
