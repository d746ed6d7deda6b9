#!/usr/bin/env python3
"""Writes the golden fixtures under tests/golden/ from the reference's conformance vectors.

Run once, in a checkout that has the reference beside it:

    python3 tests/golden/make_fixtures.py /path/to/tessera

It copies the reference's golden JSON for the hot path (spec/vectors/{blake3, encoding, hash,
transcript, pcs-streaming, sumcheck, pcs}) into gzip files here, trimmed to what the tests read.
The advice openings (spec/vectors/pcs/opening.json: honest openings with their witness, combined
rows, drawn columns and multiproofs, and the rejections a verifier must return) are copied whole. For
sumcheck stages whose tables the JSON does not record (more than 5 variables), it runs the
reference's own stdlib-Python oracle (spec/vectors/sumcheck/generate.py) and records where each
stage's tables start in its SplitMix64 stream, so the tests regenerate the tables exactly; the
script checks that rerun against the JSON before writing anything. The tree-level batches
(product trees, product forests and LogUp leaf stages, every level record) are copied whole.

The tests read only the files this script writes; nothing reads the reference at test time.
"""
from __future__ import annotations

import gzip
import importlib.util
import json
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent


def load(path: Path):
    with open(path) as f:
        return json.load(f)


def write(name: str, obj) -> None:
    data = json.dumps(obj, separators=(",", ":")).encode()
    with gzip.GzipFile(HERE / name, "wb", mtime=0) as f:
        f.write(data)
    print(f"wrote {name}: {len(data)} bytes of JSON")


def sumcheck_offsets(ref: Path, golden: dict) -> list:
    """Reruns the reference's sumcheck oracle over its sessions, recording the SplitMix64 word
    count at which each stage starts drawing its tables."""
    vec = ref / "spec" / "vectors"
    sys.path.insert(0, str(vec / "sumcheck"))
    spec = importlib.util.spec_from_file_location("tessera_sumcheck_oracle", vec / "sumcheck" / "generate.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)

    counter = {"words": 0}
    original_word = mod.Inputs.word

    def word(self):
        counter["words"] += 1
        return original_word(self)

    mod.Inputs.word = word
    offsets = []
    original_stage = mod.prove_stage

    def prove_stage(t, rng, prefix, degree, shapes):
        offsets.append(counter["words"])
        return original_stage(t, rng, prefix, degree, shapes)

    mod.prove_stage = prove_stage
    rng = mod.Inputs(mod.SEED)
    # The sessions of the oracle's main(), in its order: their shapes are the vectors' data.
    defs = [(f"single instances, products of {d} table{'s' * (d > 1)} on 0 to 12 variables",
             [(f"stage/{n}", d, [(n, d)]) for n in mod.SINGLE_VARS]) for d in mod.SINGLE_FACTORS]
    defs += [
        ("a batch of 3, 7 and 12 variables", [("stage/0", 3, [(3, 3), (7, 2), (12, 3)])]),
        ("a batch of 12, 3, 7 and 0 variables, products of 2, 4, 1 and 3 tables",
         [("stage/5", 4, [(12, 2), (3, 4), (7, 1), (0, 3)])]),
        ("a batch of equal sizes, without padding", [("stage/1", 2, [(5, 2), (5, 2), (5, 1)])]),
        ("batches of n_max = 0, then of a single instance, on one transcript",
         [("stage/0", 3, [(0, 1), (0, 2), (0, 3)]), ("stage/1", 2, [(6, 2)]), ("stage/2", 1, [(0, 1)])]),
        ("degrees 5 to 7: products of 5, 6 and 7 tables, then a batch of degree 7",
         [("stage/0", 5, [(3, 5)]), ("stage/1", 6, [(3, 6)]), ("stage/2", 7, [(3, 7)]),
          ("stage/3", 7, [(4, 7), (2, 3), (0, 1)])]),
    ]
    sessions = [mod.session(rng, name, stages) for name, stages in defs]
    if sessions != golden["sessions"]:
        raise SystemExit("the rerun of the reference's sumcheck oracle differs from sumcheck.json")
    return offsets, mod.SEED


def main() -> None:
    ref = Path(sys.argv[1] if len(sys.argv) > 1 else "../tessera").resolve()
    vec = ref / "spec" / "vectors"

    write("blake3.json.gz", load(vec / "blake3" / "test_vectors.json"))
    write("encoding.json.gz", load(vec / "encoding" / "encoding.json"))
    h = load(vec / "hash" / "hash.json")
    write("hash.json.gz", {k: h[k] for k in ("input_lengths", "domains", "merkle", "columns", "prover_streams")})
    write("transcript.json.gz", load(vec / "transcript" / "transcript.json"))
    s = load(vec / "pcs-streaming" / "streaming.json")
    write("streaming.json.gz", {"cases": s["cases"]})

    sc = load(vec / "sumcheck" / "sumcheck.json")
    offsets, seed = sumcheck_offsets(ref, sc)
    it = iter(offsets)
    sessions = []
    for session in sc["sessions"]:
        stages = []
        for stage in session["stages"]:
            stage = dict(stage)
            stage["table_word_offset"] = next(it)
            for inst in stage["instances"]:
                inst.pop("tables", None)  # regenerated from the stream by the tests
            stages.append(stage)
        sessions.append({"name": session["name"], "context": session["context"], "stages": stages})
    write("sumcheck.json.gz", {"seed": hex(seed), "sessions": sessions})
    # tree levels: product trees, product forests and LogUp leaf stages, with every level record
    write("trees.json.gz", {k: sc[k] for k in ("tree_batches", "forest_batches", "logup_batches")})
    op = load(vec / "pcs" / "opening.json")
    write("opening.json.gz", {k: op[k] for k in ("seed", "openings", "rejections")})


if __name__ == "__main__":
    main()
