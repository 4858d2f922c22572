"""Generates the golden .grad fixtures from the MSCEER reference itself.

Run on a machine that has the reference sources (the oracle/Makefile `ref` target
compiles oracle/_ref/libmsc_ref.so from them):

    make -C oracle ref && python tests/golden/make_golden.py [--large-only]

(--large-only keeps grad_small.npz and rewrites grad_large.json).

For every case it stores the float32 input and the bytes the reference's own
steepest_lstar pipeline (3D) or 2D gradient builder wrote with
DiscreteGradientLabeling::outputToFile.  Large cases store only the SHA-256 of the
.grad plus summary counts, and the input is regenerated from its seed.
"""
from __future__ import annotations

import ctypes
import hashlib
import json
import os
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
from msceer_gb300 import fields  # noqa: E402

REF = ROOT / "oracle" / "_ref" / "libmsc_ref.so"


def small_cases():
    cases = []
    for shape in [(4, 4, 4), (5, 5, 5), (7, 5, 3), (3, 3, 3), (2, 2, 2), (16, 16, 16), (13, 9, 11),
                  (1, 5, 5), (5, 1, 5), (5, 5, 1), (1, 1, 5), (6, 1, 1), (9, 7, 2), (33, 17, 19)]:
        for kind, levels in (("normal", None), ("quant4", 4), ("quant2", 2)):
            seed = 7 + len(cases)
            rng = np.random.default_rng(seed)
            f = rng.standard_normal(shape[::-1]).astype(np.float32)
            if levels:
                f = fields.quantized(f, levels)
            cases.append((f"3d_{'x'.join(map(str, shape))}_{kind}", f))
    for shape in [(4, 4), (5, 7), (64, 48), (2, 2), (3, 2), (1, 5), (5, 1), (130, 70)]:
        for kind, levels in (("normal", None), ("quant3", 3)):
            rng = np.random.default_rng(100 + len(cases))
            f = rng.standard_normal(shape[::-1]).astype(np.float32)
            if levels:
                f = fields.quantized(f, levels)
            cases.append((f"2d_{'x'.join(map(str, shape))}_{kind}", f))
    return cases


def run_ref(lib, f: np.ndarray) -> np.ndarray:
    f = np.ascontiguousarray(f, dtype=np.float32)
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "out.grad").encode()
        if f.ndim == 3:
            Z, Y, X = f.shape
            rc = lib.ref_steepest_lstar_3d(f.ctypes.data, X, Y, Z, 4, path, None)
        else:
            Y, X = f.shape
            rc = lib.ref_lstar_grad_2d(f.ctypes.data, X, Y, max(1, min(4, Y)), path, None)
        assert rc == 0
        return np.fromfile(path.decode(), dtype=np.uint8)


def summary(grad: np.ndarray, shape_xyz) -> dict:
    nd = len(shape_xyz)
    d = [2 * s - 1 for s in shape_xyz]
    ids = np.arange(grad.size, dtype=np.int64)
    coords = [ids % d[0], (ids // d[0]) % d[1]] + ([ids // (d[0] * d[1])] if nd == 3 else [])
    dim = sum((c & 1) for c in coords)
    crit = ((grad >> 2) & 7) == 7
    return {
        "sha256": hashlib.sha256(grad.tobytes()).hexdigest(),
        "critical_by_dim": [int((crit & (dim == k)).sum()) for k in range(nd + 1)],
        "ldir_hist": [int(((grad >> 5) == k).sum()) for k in range(4)],
        "assigned": int((grad & 1).sum()),
    }


def main():
    large_only = "--large-only" in sys.argv
    lib = ctypes.CDLL(str(REF))
    lib.ref_steepest_lstar_3d.argtypes = [ctypes.c_void_p, ctypes.c_longlong, ctypes.c_longlong,
                                          ctypes.c_longlong, ctypes.c_int, ctypes.c_char_p, ctypes.c_void_p]
    lib.ref_lstar_grad_2d.argtypes = [ctypes.c_void_p, ctypes.c_longlong, ctypes.c_longlong, ctypes.c_int,
                                      ctypes.c_char_p, ctypes.c_void_p]
    arrays = {}
    if not large_only:
        for name, f in small_cases():
            arrays[f"{name}__f"] = f
            arrays[f"{name}__grad"] = run_ref(lib, f)
        np.savez_compressed(HERE / "grad_small.npz", **arrays)

    big = {}
    # the bit-exact steepest_lstar workload: 64^3, 16 Gaussians, seed 0
    f = fields.gaussian_sum((64, 64, 64), 16, seed=0)
    g = run_ref(lib, f)
    big["gauss16_64"] = {"generator": "gaussian_sum((64,64,64), 16, seed=0)",
                         "f_sha256": hashlib.sha256(f.tobytes()).hexdigest(), **summary(g, (64, 64, 64))}
    f = fields.power_law_field((96, 80, 72), seed=3)
    g = run_ref(lib, f)
    big["k3_96x80x72"] = {"generator": "power_law_field((96,80,72), seed=3)",
                          "f_sha256": hashlib.sha256(f.tobytes()).hexdigest(), **summary(g, (96, 80, 72))}
    f = fields.power_law_field((512, 384), seed=5)
    g = run_ref(lib, f)
    big["k3_2d_512x384"] = {"generator": "power_law_field((512,384), seed=5)",
                            "f_sha256": hashlib.sha256(f.tobytes()).hexdigest(), **summary(g, (512, 384))}
    # the .grad scale workload: 512^3 and 8192^2 k^-3 fields, seed 0
    f = fields.power_law_field((512, 512, 512), seed=0)
    g = run_ref(lib, f)
    big["k3_512cubed"] = {"generator": "power_law_field((512,512,512), seed=0)",
                          "f_sha256": hashlib.sha256(f.tobytes()).hexdigest(), **summary(g, (512, 512, 512))}
    del f, g
    f = fields.power_law_field((8192, 8192), seed=0)
    g = run_ref(lib, f)
    big["k3_8192sq"] = {"generator": "power_law_field((8192,8192), seed=0)",
                        "f_sha256": hashlib.sha256(f.tobytes()).hexdigest(), **summary(g, (8192, 8192))}
    del f, g
    (HERE / "grad_large.json").write_text(json.dumps(big, indent=1) + "\n")
    print(f"wrote {len(arrays) // 2} small cases and {len(big)} large summaries")


if __name__ == "__main__":
    main()
