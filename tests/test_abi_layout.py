"""CPU check that the Python bindings' ctypes structures have the C header's layout: a C program
compiled against include/tessera_gb300.h prints each struct's size and field offsets, which must
equal the ctypes mirrors' (a field added on one side only would shift every later field)."""
import ctypes
import re
import shutil
import subprocess
from pathlib import Path

import pytest

from tessera_gb300 import _native as N

HEADER = Path(__file__).resolve().parent.parent / "include" / "tessera_gb300.h"
MIRRORS = {"tg_config": N.Config, "tg_transcript": N.TranscriptState, "tg_table": N.TableC,
           "tg_instance": N.InstanceC, "tg_commit_job": N.CommitJobC, "tg_proof_request": N.ProofRequestC,
           "tg_proof_result": N.ProofResultC, "tg_server_stats": N.ServerStatsC, "tg_leaf_gen": N.LeafGenC,
           "tg_tree": N.TreeC, "tg_tree_level_proof": N.TreeLevelProofC, "tg_sumcheck_job": N.SumcheckJobC,
           "tg_encode_tuning": N.EncodeTuningC}


def c_fields(name: str) -> list[str]:
    """The field names of `typedef struct [tag] { ... } name;` in declaration order."""
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    m = re.search(r"typedef struct\s*\w*\s*\{([^{}]*)\}\s*" + name + r"\s*;", text)
    assert m, name
    names = []
    for decl in m.group(1).split(";"):
        decl = decl.strip()
        if not decl:
            continue
        # "type a, b[2], *c": each declarator's name is its last identifier (array sizes dropped)
        for d in decl.split(","):
            names.append(re.findall(r"[A-Za-z_]\w*", re.sub(r"\[[^\]]*\]", "", d))[-1])
    return names


@pytest.fixture(scope="module")
def c_layout(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "tessera_gb300.h"', "int main(void) {"]
    for name in MIRRORS:
        offs = " ".join(f'printf(" %zu", offsetof({name}, {f}));' for f in c_fields(name))
        lines.append(f'printf("{name} %zu", sizeof({name})); {offs} printf("\\n");')
    lines += ["return 0;", "}"]
    d = tmp_path_factory.mktemp("abi")
    (d / "layout.c").write_text("\n".join(lines))
    subprocess.run([cc, "-std=c11", "-I", str(HEADER.parent), str(d / "layout.c"), "-o", str(d / "layout")], check=True)
    out = subprocess.run([str(d / "layout")], check=True, capture_output=True, text=True).stdout
    return {parts[0]: [int(x) for x in parts[1:]] for parts in (l.split() for l in out.splitlines())}


@pytest.mark.parametrize("name", list(MIRRORS))
def test_ctypes_mirror_matches_header(c_layout, name):
    mirror = MIRRORS[name]
    size, *offsets = c_layout[name]
    assert ctypes.sizeof(mirror) == size, name
    assert [getattr(mirror, f[0]).offset for f in mirror._fields_] == offsets, name
