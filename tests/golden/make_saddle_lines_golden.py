"""Generates tests/golden/saddle_lines.json and tests/golden/ondemand_modes.json from
the MSCEER reference itself.

Run where the reference sources are present (`make -C oracle ref` compiles
oracle/_ref/libmsc_ref.so from them):

    make -C oracle ref && python tests/golden/make_saddle_lines_golden.py

For every case the labels are the reference's saddle streamline digitizers
(ondemandaccurate's needASC1 / needDSC1 lines, DigitizingNumericStreamlineIntegrator3dASC /
3dDSC) at one thread on the gradient of f, over the reference's own .grad, starting
from the given cell labels; the oracle's restatement is checked equal first.  The
fixture stores the SHA-256 of the cell labels; the input is regenerated from its
generator (f_sha256 says whether a machine regenerated the same floats: the FFT-based
fields can differ in their last bits between hosts, and the streamlines with them).
ondemand_modes.json holds, per case and flags (needASC1, needDSC1, needASC2,
needDSC2), the SHA-256 of the restriction labels and of the accurate .grad the
reference's ondemandaccurate writes at one thread (the oracle checked equal first).
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

# name, field generator, which (1 ascending lines, 2 descending, 3 both), preset
# labels (None: all zero; (seed, 1 / fraction): that share of the cells labelled 1, 2, 4
# or 5 by numpy.random.default_rng(seed))
CASES = [
    ("gauss16_48_both", "gaussian_sum((48,48,48), 16, seed=0)", 3, None),
    ("gauss64_40x44x48_both_preset", "gaussian_sum((40,44,48), 64, seed=4)", 3, (7, 200)),
    ("gauss12_33x29x31_asc", "gaussian_sum((33,29,31), 12, seed=9)", 1, None),
    ("gauss12_33x29x31_dsc_preset", "gaussian_sum((33,29,31), 12, seed=9)", 2, (3, 100)),
    ("k3_24x20x18_both", "power_law_field((24,20,18), seed=2)", 3, None),
]
ERROR, ITERS, MAX_STEP = 1e-4, 4000, 0.25
MODE_CASES = [
    ("gauss12_28x26x24", "gaussian_sum((28,26,24), 12, seed=2)"),
    ("gauss32_36x32x30", "gaussian_sum((36,32,30), 32, seed=6)"),
]
MODES = [(1, 0, 0, 0), (0, 1, 0, 0), (1, 1, 1, 1), (1, 0, 1, 0), (0, 1, 0, 1), (0, 0, 1, 1)]


def preset_cells(nc: int, spec):
    cells = np.zeros(nc, np.uint8)
    if spec is None:
        return cells
    rng = np.random.default_rng(spec[0])
    idx = rng.choice(nc, nc // spec[1], replace=False)
    cells[idx] = rng.choice(np.array([1, 2, 4, 5], np.uint8), idx.size)
    return cells


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def main() -> None:
    ref = oracle_lib.load_ref()
    if ref is None or not hasattr(ref, "ref_saddle_lines_3d"):
        raise SystemExit("build the reference harness first: make -C oracle ref")
    orc = oracle_lib.load()
    out = {}
    for name, gen, which, preset in CASES:
        f = eval("fields." + gen).astype(np.float32)
        g = oracle_lib.ref_grad(ref, f)
        gt = 1e-6 * float(np.abs(f).max())
        cells = preset_cells(g.size, preset)
        want = oracle_lib.ref_saddle_lines(ref, f, which, ERROR, gt, ITERS, cells)
        got = orc.saddle_lines(f, g, which, ERROR, gt, ITERS, MAX_STEP, cells)
        assert np.array_equal(got, want), name
        out[name] = {"generator": gen, "which": which, "preset": list(preset) if preset else None,
                     "f_sha256": digest(f), "grad_sha256": digest(g), "labelled": int((want > 0).sum()),
                     "sha256": digest(want)}
        print(name, out[name]["labelled"])
    (HERE / "saddle_lines.json").write_text(json.dumps(out, indent=1) + "\n")
    modes = {}
    for name, gen in MODE_CASES:
        f = eval("fields." + gen).astype(np.float32)
        g = oracle_lib.ref_grad(ref, f)
        gt = 1e-6 * float(np.abs(f).max())
        entry = {"generator": gen, "f_sha256": digest(f), "grad_sha256": digest(g), "modes": {}}
        for flags in MODES:
            rr, rg = oracle_lib.ref_ondemand_modes(ref, f, flags, ERROR, gt, ITERS)
            orr, org = orc.ondemand_grad(f, g, flags, ERROR, gt, ITERS, MAX_STEP)
            assert np.array_equal(orr, rr) and np.array_equal(org, rg), (name, flags)
            entry["modes"]["".join(map(str, flags))] = {"restricted": int((rr > 0).sum()), "restrict_sha256": digest(rr),
                                                        "grad_sha256": digest(rg)}
        modes[name] = entry
        print(name, {k: v["restricted"] for k, v in entry["modes"].items()})
    (HERE / "ondemand_modes.json").write_text(json.dumps(modes, indent=1) + "\n")


if __name__ == "__main__":
    main()
