"""INTEGRATION.md's C++ snippets compiled against the reference's own headers and sources
(where the reference is present on this machine) and run, with the library calls
served by a CPU stand-in over the oracle (tests/msc_gpu_stub.c), so no GPU is needed:
  * the .grad the reference's DiscreteGradientLabeling::outputToFile writes from the
    array msc_steepest_lstar_host filled equals the reference's own steepest_lstar
    output byte for byte;
  * the MorseSmaleComplexBasic built from msc_ms_graph_3d's arrays equals the
    reference's own ComputeFromGrad node for node and arc for arc, list links
    included."""
import os
import subprocess
from pathlib import Path

import numpy as np
import pytest

import oracle_lib
from msceer_gb300 import fields

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
REF = Path(os.environ.get("MSC_REF_ROOT", "/root/reference"))


needs_ref = pytest.mark.skipif(not (REF / "include" / "gi_discrete_gradient_labeling.h").exists(),
                               reason="the reference sources are not on this machine")


def _build(tmp_path, source):
    ref = oracle_lib.load_ref()
    if ref is None:
        pytest.skip("the reference harness is not built")
    oracle_lib.load()
    stub = tmp_path / "libmsc_gpu.so"
    if not stub.exists():
        subprocess.run(["gcc", "-O2", "-shared", "-fPIC", "-o", str(stub), str(HERE / "msc_gpu_stub.c"),
                        str(oracle_lib.ORACLE_SO), f"-Wl,-rpath,{oracle_lib.ORACLE_SO.parent}"], check=True)
    exe = tmp_path / Path(source).stem
    srcs = [str(REF / "src" / s) for s in ("gi_regular_grid.cxx", "gi_regular_grid_trilinear_function.cxx",
                                           "gi_topological_regular_grid.cxx")]
    subprocess.run(["g++", "-O1", "-std=c++17", "-fopenmp", "-w", f"-I{REF / 'include'}", f"-I{ROOT / 'include'}",
                    str(HERE / source), *srcs, "-o", str(exe), f"-L{tmp_path}", "-lmsc_gpu",
                    f"-Wl,-rpath,{tmp_path}"], check=True)
    return ref, exe


@needs_ref
def test_snippet_against_reference(tmp_path):
    ref, exe = _build(tmp_path, "integration_snippet.cpp")
    f = fields.gaussian_sum((24, 20, 16), 6, seed=4)
    raw = tmp_path / "vol.raw"
    f.tofile(raw)
    out = tmp_path / "out.grad"
    res = subprocess.run([str(exe), "24", "20", "16", str(raw), str(out)], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    got = np.fromfile(out, dtype=np.uint8)
    assert np.array_equal(got, oracle_lib.ref_grad(ref, f))


@needs_ref
def test_ms_graph_snippet_against_reference(tmp_path):
    ref, exe = _build(tmp_path, "integration_ms_graph.cpp")
    f = fields.power_law_field((20, 18, 22), seed=7)   # X, Y, Z
    raw = tmp_path / "vol.raw"
    f.tofile(raw)
    grad = tmp_path / "vol.grad"
    oracle_lib.ref_grad(ref, f).tofile(grad)
    Z, Y, X = f.shape
    res = subprocess.run([str(exe), str(X), str(Y), str(Z), str(raw), str(grad)], capture_output=True, text=True)
    assert res.returncode == 0, (res.returncode, res.stdout[-2000:])
    assert "arcs equal" in res.stdout
