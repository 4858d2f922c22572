"""The CPU oracle against the reference's own outputs (no GPU needed)."""
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

import oracle_lib
from msceer_gb300 import fields

GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.mark.parametrize("case", oracle_lib.load_golden_small(), ids=lambda c: c[0])
def test_oracle_matches_reference_golden(oracle, case):
    name, f, want = case
    got = oracle.grad(f, nthreads=2)
    assert np.array_equal(got, want), oracle_lib.describe_mismatch(got, want, f.shape[::-1])


def _regenerate(spec):
    return eval("fields." + spec["generator"], {"fields": fields})


@pytest.mark.parametrize("key", ["gauss16_64", "k3_96x80x72", "k3_2d_512x384"])
def test_oracle_matches_reference_large_hash(oracle, key):
    spec = json.loads((GOLDEN / "grad_large.json").read_text())[key]
    f = _regenerate(spec)
    if hashlib.sha256(f.tobytes()).hexdigest() != spec["f_sha256"]:
        pytest.skip("this platform's generator output differs from the fixture's input")
    g = oracle.grad(f)
    assert hashlib.sha256(g.tobytes()).hexdigest() == spec["sha256"]


def test_oracle_stages_compose(oracle):
    f = fields.power_law_field((24, 20, 18), seed=11)
    g = oracle.pairs(f)
    g = oracle.ldir(g, f.shape[::-1])
    dims = f.shape[::-1]
    oracle.lib.oracle_flag_3d(*dims, g.ctypes.data)
    assert np.array_equal(g, oracle.grad(f))


def test_oracle_thread_count_invariant(oracle):
    f = fields.quantized(fields.power_law_field((40, 33, 29), seed=2), 5)
    assert np.array_equal(oracle.grad(f, nthreads=1), oracle.grad(f, nthreads=4))


def test_comparison_detects_planted_mistake(oracle):
    """Plant a one-bit mistake in the oracle's output: the parity check must see it."""
    _, f, want = oracle_lib.load_golden_small()[0]
    got = oracle.grad(f)
    got[len(got) // 2] ^= 0x04
    assert not np.array_equal(got, want)
    assert "1 cells differ" in oracle_lib.describe_mismatch(got, want, f.shape[::-1])


def test_oracle_against_compiled_reference_random():
    ref = oracle_lib.load_ref()
    if ref is None:
        pytest.skip("reference sources not on this machine")
    orc = oracle_lib.load()
    rng = np.random.default_rng(1234)
    for trial in range(12):
        shape = tuple(int(s) for s in rng.integers(2, 14, size=3))
        f = rng.standard_normal(shape[::-1]).astype(np.float32)
        if trial % 2:
            f = fields.quantized(f, int(rng.integers(2, 6)))
        want = oracle_lib.ref_grad(ref, f)
        got = orc.grad(f)
        assert np.array_equal(got, want), (shape, oracle_lib.describe_mismatch(got, want, shape))
    for trial in range(6):
        shape = tuple(int(s) for s in rng.integers(2, 40, size=2))
        f = fields.quantized(rng.standard_normal(shape[::-1]).astype(np.float32), 3)
        want = oracle_lib.ref_grad(ref, f)
        assert np.array_equal(orc.grad(f), want), shape


def test_central_diff_oracle_against_reference(oracle):
    ref = oracle_lib.load_ref()
    if ref is None:
        pytest.skip("reference sources not on this machine")
    for shape in [(5, 4, 3), (1, 7, 2), (33, 20, 17), (2, 2, 2)]:
        f = fields.power_law_field(shape, seed=4)
        f.flat[::7] *= -1.0
        want = np.zeros(f.shape + (3,))
        ref.ref_central_diff_3d(f.ctypes.data, *shape, want.ctypes.data)
        got = oracle.central_diff(f)
        assert np.array_equal(got.view(np.uint64), want.view(np.uint64)), shape


def test_central_diff_oracle_boundary_zero(oracle):
    f = fields.gaussian_sum((9, 8, 7), 3, seed=1)
    g = oracle.central_diff(f)
    assert (g[0, :, :, 2] == 0).all() and (g[-1, :, :, 2] == 0).all()
    assert (g[:, :, 0, 0] == 0).all() and (g[:, :, -1, 0] == 0).all()
    x = 3
    assert g[4, 4, x, 0] == 0.5 * float(f[4, 4, x + 1]) - 0.5 * float(f[4, 4, x - 1])


def test_label_oracle_against_compiled_reference(oracle):
    """The FP64 labeling oracle equals the single-thread reference at every stage."""
    ref = oracle_lib.load_ref()
    if ref is None:
        pytest.skip("reference sources not on this machine")
    for f in (fields.gaussian_sum((14, 12, 10), 4, seed=1), fields.power_law_field((16, 15, 13), seed=2),
              fields.gaussian_sum((30, 28, 26), 8, seed=3)):
        gt = 1e-6 * float(np.abs(f).max())
        want = oracle_lib.ref_labels(ref, f, 1e-4, gt, 4000, 0.0)
        got = oracle.labels(f, oracle.grad(f), 1e-4, gt, 4000, 0.25, 0.0)
        for k in want:
            assert np.array_equal(got[k], want[k]), (f.shape, k, int((got[k] != want[k]).sum()))


@pytest.mark.parametrize("make", [lambda: fields.gaussian_sum((40, 36, 32), 8, seed=5),
                                  lambda: fields.power_law_field((32, 30, 28), seed=6)], ids=["gauss40", "k3_32"])
def test_conforming_grad_oracle_against_reference(oracle, make):
    """ondemandaccurate's accurate 3-manifold .grad: the oracle's restriction labels and
    constrained re-pairing, fed the reference's own final labels, give the reference's
    restriction labels and .grad byte for byte."""
    ref = oracle_lib.load_ref()
    if ref is None:
        pytest.skip("the reference is not compiled on this machine")
    f = make()
    gt = 1e-6 * float(np.abs(f).max())
    want = oracle_lib.ref_ondemand(ref, f, 1e-4, gt, 4000, 0.0)
    restrict = oracle.boundary_labels(f, want["asc"], want["dsc"])
    assert np.array_equal(restrict, want["restrict"]), int((restrict != want["restrict"]).sum())
    assert (restrict > 0).any()
    base = oracle.grad(f)
    got = oracle.conform(f, restrict, base)
    assert np.array_equal(got, want["grad"]), oracle_lib.describe_mismatch(got, want["grad"], f.shape[::-1])
    assert not np.array_equal(got, base)   # the re-pairing changed something


MS_GRAPH_CASES = json.loads((GOLDEN / "ms_graph.json").read_text())


def _digests(graph):
    return {k: hashlib.sha256(np.ascontiguousarray(v).tobytes()).hexdigest() for k, v in graph.items()}


@pytest.mark.parametrize("key", sorted(MS_GRAPH_CASES))
def test_ms_graph_oracle_against_golden(oracle, key):
    """MorseSmaleComplexBasic::ComputeFromGrad restated: nodes and arcs (with
    multiplicity and order) equal the reference's on its own .grad, by SHA-256."""
    spec = MS_GRAPH_CASES[key]
    f = _regenerate(spec).astype(np.float32)
    g = oracle.grad(f)
    assert hashlib.sha256(g.tobytes()).hexdigest() == spec["grad_sha256"]
    got = oracle.ms_graph(f, g, spec["build_arcs"])
    assert (got["node_cell"].size, got["arc_lower"].size) == (spec["nodes"], spec["arcs"])
    d = _digests(got)
    same_f = hashlib.sha256(f.tobytes()).hexdigest() == spec["f_sha256"]
    keys = spec["sha256"] if same_f else [k for k in spec["sha256"] if k not in ("node_value", "arc_persistence")]
    assert {k: d[k] for k in keys} == {k: spec["sha256"][k] for k in keys}


@pytest.mark.parametrize("build", [(1, 0, 1), (1, 1, 1), (0, 1, 0)])
def test_ms_graph_oracle_against_reference(oracle, build):
    ref = oracle_lib.load_ref()
    if ref is None:
        pytest.skip("the reference is not compiled on this machine")
    for f in (fields.power_law_field((30, 26, 22), seed=11), fields.gaussian_sum((28, 24, 20), 12, seed=12)):
        g = oracle.grad(f)
        got = oracle.ms_graph(f, g, build)
        want = oracle_lib.ref_ms_graph(ref, f, g, build)
        for k in want:
            assert np.array_equal(got[k], want[k]), k


SADDLE_LINES_CASES = json.loads((GOLDEN / "saddle_lines.json").read_text())


def _preset_cells(nc, spec):
    cells = np.zeros(nc, np.uint8)
    if spec is None:
        return cells
    rng = np.random.default_rng(spec[0])
    idx = rng.choice(nc, nc // spec[1], replace=False)
    cells[idx] = rng.choice(np.array([1, 2, 4, 5], np.uint8), idx.size)
    return cells


@pytest.mark.parametrize("key", sorted(SADDLE_LINES_CASES))
def test_saddle_lines_oracle_against_golden(oracle, key):
    """ondemandaccurate's saddle streamline digitizers (needASC1 / needDSC1) restated:
    the cell labels equal the reference's, by SHA-256 (on the same floats of f)."""
    spec = SADDLE_LINES_CASES[key]
    f = _regenerate(spec).astype(np.float32)
    g = oracle.grad(f)
    assert hashlib.sha256(g.tobytes()).hexdigest() == spec["grad_sha256"]
    if hashlib.sha256(f.tobytes()).hexdigest() != spec["f_sha256"]:
        pytest.skip("this host regenerates other floats for the field (FFT); the streamlines follow them")
    gt = 1e-6 * float(np.abs(f).max())
    got = oracle.saddle_lines(f, g, spec["which"], 1e-4, gt, 4000, 0.25, _preset_cells(g.size, spec["preset"]))
    assert int((got > 0).sum()) == spec["labelled"]
    assert hashlib.sha256(got.tobytes()).hexdigest() == spec["sha256"]


@pytest.mark.parametrize("which", [1, 2, 3])
def test_saddle_lines_oracle_against_reference(oracle, which):
    ref = oracle_lib.load_ref()
    if ref is None or not hasattr(ref, "ref_saddle_lines_3d"):
        pytest.skip("the reference is not compiled on this machine")
    for f, preset in ((fields.power_law_field((30, 26, 22), seed=13), None),
                      (fields.gaussian_sum((28, 24, 20), 10, seed=14), (5, 50))):
        g = oracle.grad(f)
        gt = 1e-6 * float(np.abs(f).max())
        cells = _preset_cells(g.size, preset)
        got = oracle.saddle_lines(f, g, which, 1e-4, gt, 4000, 0.25, cells)
        want = oracle_lib.ref_saddle_lines(ref, f, which, 1e-4, gt, 4000, cells)
        assert (want > 0).sum() > 0
        assert np.array_equal(got, want), int((got != want).sum())


ONDEMAND_MODE_CASES = json.loads((GOLDEN / "ondemand_modes.json").read_text())


@pytest.mark.parametrize("key", sorted(ONDEMAND_MODE_CASES))
def test_ondemand_modes_oracle_against_golden(oracle, key):
    """ondemandaccurate's accurate .grad for every combination of needASC1 / needDSC1 /
    needASC2 / needDSC2 in the fixture: restriction labels and .grad equal the
    reference's, by SHA-256 (on the same floats of f)."""
    spec = ONDEMAND_MODE_CASES[key]
    f = _regenerate(spec).astype(np.float32)
    g = oracle.grad(f)
    assert hashlib.sha256(g.tobytes()).hexdigest() == spec["grad_sha256"]
    if hashlib.sha256(f.tobytes()).hexdigest() != spec["f_sha256"]:
        pytest.skip("this host regenerates other floats for the field; the streamlines follow them")
    gt = 1e-6 * float(np.abs(f).max())
    for flags, want in spec["modes"].items():
        restrict, grad = oracle.ondemand_grad(f, g, [int(c) for c in flags], 1e-4, gt, 4000, 0.25)
        assert int((restrict > 0).sum()) == want["restricted"], flags
        assert hashlib.sha256(restrict.tobytes()).hexdigest() == want["restrict_sha256"], flags
        assert hashlib.sha256(grad.tobytes()).hexdigest() == want["grad_sha256"], flags


@pytest.mark.parametrize("flags", [(1, 0, 0, 0), (0, 1, 0, 0), (1, 1, 1, 1), (0, 1, 1, 0)])
def test_ondemand_modes_oracle_against_reference(oracle, flags):
    ref = oracle_lib.load_ref()
    if ref is None or not hasattr(ref, "ref_ondemand_modes_3d"):
        pytest.skip("the reference is not compiled on this machine")
    f = fields.power_law_field((26, 22, 20), seed=17)
    g = oracle.grad(f)
    gt = 1e-6 * float(np.abs(f).max())
    restrict, grad = oracle.ondemand_grad(f, g, flags, 1e-4, gt, 4000, 0.25)
    want_r, want_g = oracle_lib.ref_ondemand_modes(ref, f, flags, 1e-4, gt, 4000)
    assert (want_r > 0).sum() > 0
    assert np.array_equal(restrict, want_r), int((restrict != want_r).sum())
    assert np.array_equal(grad, want_g), oracle_lib.describe_mismatch(grad, want_g, f.shape[::-1])
