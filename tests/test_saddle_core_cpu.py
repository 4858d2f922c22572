"""The saddle streamline digitizers' parallel form, compiled for the host, against the
one-thread oracle and the reference's fixtures (no GPU).

tests/saddle_core_host.cpp drives msceer_gb300/csrc/saddle_core.cuh -- the per-streamline
code a kernel runs: label-free integration into per-voxel-step records, then rounds of
claims and walks until no claim changes.  The cell labels must equal the one-thread
result byte for byte, however the streamlines' ends depend on one another."""
import ctypes
import hashlib
import json
import subprocess
from pathlib import Path

import numpy as np
import pytest

from msceer_gb300 import fields

HERE = Path(__file__).resolve().parent
GOLDEN = HERE / "golden"
CASES = json.loads((GOLDEN / "saddle_lines.json").read_text())
_VP, _I64 = ctypes.c_void_p, ctypes.c_int64


@pytest.fixture(scope="module")
def core(tmp_path_factory):
    out = tmp_path_factory.mktemp("saddle_core") / "libsaddlecore.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-shared", "-fPIC", "-o", str(out),
                    str(HERE / "saddle_core_host.cpp")], check=True)
    lib = ctypes.CDLL(str(out))
    lib.core_saddle_lines_3d.argtypes = [_VP, _VP, _VP, _I64, _I64, _I64, ctypes.c_int, ctypes.c_float,
                                         ctypes.c_float, ctypes.c_double, ctypes.c_int, ctypes.c_int, _VP, _VP]
    return lib


def preset_cells(nc, spec):
    """The fixtures' preset labels: nc // spec[1] random cells labelled 1, 2, 4 or 5."""
    cells = np.zeros(nc, np.uint8)
    if spec is None:
        return cells
    rng = np.random.default_rng(spec[0])
    idx = rng.choice(nc, nc // spec[1], replace=False)
    cells[idx] = rng.choice(np.array([1, 2, 4, 5], np.uint8), idx.size)
    return cells


def run_core(core, f, g, which, cells, zeroed=None, budget=0):
    """(cells after the lines, [streamlines, recorded steps, kept steps, rounds, pieces]);
    budget 0 traces the streamlines whole before the rounds, b > 0 in growing pieces."""
    out = np.array(cells, dtype=np.uint8, copy=True)
    stats = np.zeros(5, np.int64)
    gt = 1e-6 * float(np.abs(f).max())
    zp = None if zeroed is None else zeroed.ctypes.data
    rc = core.core_saddle_lines_3d(f.ctypes.data, g.ctypes.data, zp, *f.shape[::-1], which, 1e-4, gt, 0.25, 4000,
                                   budget, out.ctypes.data, stats.ctypes.data)
    assert rc == 0
    return out, stats


@pytest.mark.parametrize("budget", [0, 2])
@pytest.mark.parametrize("key", sorted(CASES))
def test_parallel_lines_against_golden(core, oracle, key, budget):
    spec = CASES[key]
    f = eval("fields." + spec["generator"], {"fields": fields}).astype(np.float32)
    if hashlib.sha256(f.tobytes()).hexdigest() != spec["f_sha256"]:
        pytest.skip("this host regenerates other floats for the field (FFT); the streamlines follow them")
    g = oracle.grad(f)
    got, stats = run_core(core, f, g, spec["which"], preset_cells(g.size, spec["preset"]), budget=budget)
    assert int((got > 0).sum()) == spec["labelled"]
    assert hashlib.sha256(got.tobytes()).hexdigest() == spec["sha256"]
    assert stats[3] >= 2 and stats[2] <= stats[1]


@pytest.mark.parametrize("which", [1, 2, 3])
@pytest.mark.parametrize("case", ["k3", "gauss_preset", "k3_preset_dense"])
def test_parallel_lines_against_oracle(core, oracle, case, which):
    if case == "k3":
        f, preset = fields.power_law_field((30, 26, 22), seed=13), None
    elif case == "gauss_preset":
        f, preset = fields.gaussian_sum((28, 24, 20), 10, seed=14), (5, 50)
    else:  # a label on every fourth cell: most streamlines end within a few steps
        f, preset = fields.power_law_field((26, 22, 30), seed=21), (8, 4)
    f = f.astype(np.float32)
    g = oracle.grad(f)
    cells = preset_cells(g.size, preset)
    gt = 1e-6 * float(np.abs(f).max())
    want = oracle.saddle_lines(f, g, which, 1e-4, gt, 4000, 0.25, cells)
    got, stats = run_core(core, f, g, which, cells)
    assert (want != cells).sum() > 0
    assert np.array_equal(got, want), int((got != want).sum())
    assert stats[0] > 0 and stats[3] >= 2
    # traced in pieces (4, 8, 16, ... voxel steps, continued only where a walk runs past
    # its records): the same labels from fewer recorded steps
    lazy, ls = run_core(core, f, g, which, cells, budget=4)
    assert np.array_equal(lazy, want), int((lazy != want).sum())
    assert ls[1] <= stats[1] and ls[2] == stats[2] and ls[4] >= ls[0]


@pytest.mark.parametrize("which", [1, 2, 3])
def test_parallel_lines_zeroed_gradient(core, oracle, which):
    """The gradient zero at a set of vertices (as the integrations before the lines leave
    it at their seeds): equal to the oracle on the same zeroed set, and different from
    the plain gradient's lines."""
    f = fields.power_law_field((24, 22, 20), seed=5).astype(np.float32)
    g = oracle.grad(f)
    cells = np.zeros(g.size, np.uint8)
    bits = np.zeros(((f.size + 31) // 32 + 1) * 32, bool)
    bits[np.random.default_rng(1).choice(f.size, f.size // 16, replace=False)] = True
    zeroed = np.packbits(bits, bitorder="little").view(np.uint32).copy()
    gt = 1e-6 * float(np.abs(f).max())
    want = oracle.saddle_lines(f, g, which, 1e-4, gt, 4000, 0.25, cells, zeroed)
    got, _ = run_core(core, f, g, which, cells, zeroed)
    assert np.array_equal(got, want), int((got != want).sum())
    plain, _ = run_core(core, f, g, which, cells)
    assert not np.array_equal(plain, got)
