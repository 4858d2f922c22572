"""Generates tests/golden/ms_graph.json from the MSCEER reference itself.

Run where the reference sources are present (`make -C oracle ref` compiles
oracle/_ref/libmsc_ref.so from them):

    make -C oracle ref && python tests/golden/make_ms_graph_golden.py

For every case the .grad is the reference's own steepest_lstar output and the graph is
the reference's MorseSmaleComplexBasic::ComputeFromGrad on it, with the given arc build
flags and no arc geometry (extractmsc's setup).  The fixture stores the node and arc
counts and the SHA-256 of every array; the input is regenerated from its generator
(f_sha256 says whether a machine regenerated the same floats: the FFT-based fields can
differ in their last bits between hosts, which moves the node values but not the
.grad, the nodes or the arcs).
"""
from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))
from msceer_gb300 import fields  # noqa: E402,F401

import oracle_lib  # noqa: E402

CASES = [
    ("gauss16_64_extractmsc", "gaussian_sum((64,64,64), 16, seed=0)", (1, 0, 1)),
    ("gauss16_64_all", "gaussian_sum((64,64,64), 16, seed=0)", (1, 1, 1)),
    ("k3_36x40x48_all", "power_law_field((36,40,48), seed=3)", (1, 1, 1)),
    ("k3_9x12x1_all", "power_law_field((9,12,1), seed=4)", (1, 1, 1)),
    ("k3_15x1x20_all", "power_law_field((15,1,20), seed=5)", (1, 1, 1)),
]


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def main() -> None:
    ref = oracle_lib.load_ref()
    if ref is None:
        raise SystemExit("build the reference harness first: make -C oracle ref")
    out = {}
    for name, gen, build in CASES:
        f = eval("fields." + gen).astype(np.float32)
        g = oracle_lib.ref_grad(ref, f)
        r = oracle_lib.ref_ms_graph(ref, f, g, build)
        out[name] = {"generator": gen, "build_arcs": list(build), "f_sha256": digest(f), "grad_sha256": digest(g),
                     "nodes": int(r["node_cell"].size), "arcs": int(r["arc_lower"].size),
                     "sha256": {k: digest(v) for k, v in r.items()}}
        print(name, out[name]["nodes"], out[name]["arcs"])
    (HERE / "ms_graph.json").write_text(json.dumps(out, indent=1) + "\n")


if __name__ == "__main__":
    main()
