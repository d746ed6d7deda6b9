"""Builds libtessera_gb300.so for sm_103a with nvcc, in-tree (tessera_gb300/_build/).

Each translation unit compiles in parallel (one -gencode, so a few seconds each), then one link.
The CUDA runtime is linked statically, so the library needs only the driver at run time.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT = PKG / "_build"
LIB = OUT / "libtessera_gb300.so"
SOURCES = ["lde.cu", "hash.cu", "host.cu", "capi.cu", "sumcheck.cu", "level.cu", "noalloc.cu", "peaks.cu", "batch.cu", "workload.cu", "serve.cu", "opening.cu", "trees.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
         "-I", str(PKG.parent / "include")]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is needed to build libtessera_gb300")


def _compile(src: Path, obj: Path, extra: list[str]) -> None:
    cmd = [nvcc(), *ARCH, *FLAGS, *extra, "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stdout}\n{r.stderr}")


def up_to_date() -> bool:
    if not LIB.exists():
        return False
    t = LIB.stat().st_mtime
    deps = list(CSRC.glob("*")) + [PKG.parent / "include" / "tessera_gb300.h", Path(__file__)]
    return all(p.stat().st_mtime <= t for p in deps)


def build(force: bool = False, extra: list[str] | None = None) -> Path:
    """Compiles the library if any source is newer than it; returns its path."""
    if not force and up_to_date():
        return LIB
    OUT.mkdir(exist_ok=True)
    extra = list(extra or [])
    objs = [OUT / (Path(s).stem + ".o") for s in SOURCES]
    with cf.ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 4)) as ex:
        futs = [ex.submit(_compile, CSRC / s, o, extra) for s, o in zip(SOURCES, objs)]
        for f in futs:
            f.result()
    tmp = OUT / "libtessera_gb300.so.tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-cudart", "static", "-o", str(tmp), *map(str, objs)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
