"""The ondemandaccurate command line (msceer_gb300/bin/ondemandaccurate) against the
oracle: same argv as ondemandaccurate/ondemandaccurate.cxx:158-185, the .grad it
writes, its timing file, its debug dumps and its exit status."""
import os
import subprocess

import numpy as np
import pytest

from msceer_gb300 import build, fields

pytestmark = pytest.mark.gpu


def run_cli(tmp_path, f, need_asc3, need_dsc3, extra=(), need_asc1=0):
    build.build_cli()
    exe = build.BIN / "ondemandaccurate"
    raw = tmp_path / "vol.raw"
    f.tofile(raw)
    X, Y, Z = f.shape[::-1]
    gt = 1e-6 * float(np.abs(f).max())
    env = dict(os.environ, MSC_MAX_STEP_IN_GRID_CELLS="0.25")
    args = [str(exe), str(X), str(Y), str(Z), str(raw), "1e-4", repr(gt), "4000", str(need_asc1), "0",
            str(need_asc3), str(need_dsc3), "0", *extra]
    res = subprocess.run(args, capture_output=True, text=True, cwd=tmp_path, env=env)
    return res, raw


def test_accurate_3_manifolds(gpu, oracle, tmp_path):
    """needASC2 = needDSC2 = 1 on a field where the GPU labels and the oracle's lead to
    the same restriction labels: the .grad equals the oracle's conforming .grad (itself
    the reference's), byte for byte; the debug dumps hold the ascending labels."""
    f = fields.gaussian_sum((40, 36, 32), 8, seed=5)
    res, raw = run_cli(tmp_path, f, 1, 1, extra=["8", "1"])
    assert res.returncode == 1, res.stdout + res.stderr
    gt = 1e-6 * float(np.abs(f).max())
    base = oracle.grad(f)
    lab = oracle.labels(f, base, 1e-4, gt, 4000, 0.25, 0.0)
    want = oracle.conform(f, oracle.boundary_labels(f, lab["asc"], lab["dsc"]), base)
    got = np.fromfile(str(raw) + ".grad", dtype=np.uint8)
    assert np.array_equal(got, want), int((got != want).sum())
    assert (tmp_path / "vol.raw.008.gtime.txt").read_text().splitlines()[0].startswith("Topological Robins0 ")
    cleaned = np.fromfile(tmp_path / "newintegrator_cleaned_asc.raw", dtype=np.int32)
    assert float((cleaned != lab["asc"]).mean()) <= 1e-3
    terminal = np.fromfile(tmp_path / "extremal_asc.raw", dtype=np.int32)
    assert np.array_equal(terminal, lab["asc_terminal"])
    assert np.fromfile(tmp_path / "boundaries_79x71x63.raw", dtype=np.uint8).size == got.size


def test_no_accuracy_requested_writes_the_lower_star_grad(gpu, oracle, tmp_path):
    f = fields.power_law_field((30, 26, 22), seed=2)
    res, raw = run_cli(tmp_path, f, 0, 0)
    assert res.returncode == 1, res.stdout + res.stderr
    assert np.array_equal(np.fromfile(str(raw) + ".grad", dtype=np.uint8), oracle.grad(f))
    assert (tmp_path / "vol.raw.-01.gtime.txt").exists()  # the reference's "%03d" of the default -1


def test_saddle_line_modes_refused(gpu, tmp_path):
    f = fields.gaussian_sum((16, 16, 16), 2, seed=1)
    res, raw = run_cli(tmp_path, f, 0, 0, need_asc1=1)
    assert res.returncode == 2
    assert "not provided" in res.stderr
    assert not os.path.exists(str(raw) + ".grad")
