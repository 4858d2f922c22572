"""The C ABI library: loads, exports every declared symbol, validates arguments.
No compute call here needs a GPU."""
import ctypes
import re
import subprocess
from pathlib import Path

import pytest

from msceer_gb300 import _lib, build

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def lib():
    build.build_library()
    return _lib.load()


def declared_symbols():
    text = "\n".join(p.read_text() for p in sorted((ROOT / "include").glob("*.h")))
    return sorted(set(re.findall(r"^\s*(?:int|int64_t|void|const char\*)\s+(msc_\w+)\s*\(", text, re.M)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "msc_lower_star_grad_3d" in syms and "msc_steepest_lstar_host" in syms
    assert "msc_triage_labels_3d" in syms and "msc_labels_last_stats" in syms
    assert len(syms) >= 12


def test_library_exports_every_declared_symbol(lib):
    nm = subprocess.run(["nm", "-D", "--defined-only", str(_lib.lib_path())], capture_output=True, text=True,
                        check=True).stdout
    exported = set(re.findall(r"\bT (msc_\w+)", nm))
    for s in declared_symbols():
        assert s in exported, s
        assert s in _lib.SIGNATURES, s


def test_num_cells(lib):
    assert lib.msc_num_cells_3d(_lib.dims_arg((64, 64, 64))) == 127 ** 3
    assert lib.msc_num_cells_3d(_lib.dims_arg((512, 512, 512))) == 1023 ** 3
    assert lib.msc_num_cells_2d(_lib.dims_arg((8192, 8192))) == 16383 ** 2
    assert lib.msc_num_cells_3d(_lib.dims_arg((0, 4, 4))) == -1
    assert lib.msc_num_cells_2d(_lib.dims_arg((-3, 4))) == -1


def test_argument_errors_before_any_device_work(lib):
    buf = ctypes.create_string_buffer(64)
    rc = lib.msc_lower_star_grad_3d(ctypes.c_void_p(ctypes.addressof(buf)), _lib.dims_arg((0, 2, 2)),
                                    ctypes.c_void_p(ctypes.addressof(buf)), None)
    assert rc == -1
    assert b"dims" in lib.msc_last_error_string()
    rc = lib.msc_lower_star_grad_3d(None, _lib.dims_arg((2, 2, 2)), None, None)
    assert rc == -2
    with pytest.raises(_lib.MscError) as e:
        _lib.check(rc, "msc_lower_star_grad_3d")
    assert "MSC_ERR_NULL_POINTER" in str(e.value)


def test_saddle_lines_argument_errors_before_any_device_work(lib):
    """msc_saddle_lines_3d rejects bad dims, null buffers and a bad `which` before it
    touches the device."""
    buf = ctypes.create_string_buffer(64)
    b = ctypes.c_void_p(ctypes.addressof(buf))
    p = _lib.IntegParams(1e-4, 1e-6, 4000, 0.25, 0.0, 0)
    sl = lib.msc_saddle_lines_3d
    assert sl(b, b, None, _lib.dims_arg((1, 4, 4)), 3, ctypes.byref(p), b, None, None) == -1
    assert sl(None, b, None, _lib.dims_arg((4, 4, 4)), 3, ctypes.byref(p), b, None, None) == -2
    assert sl(b, b, None, _lib.dims_arg((4, 4, 4)), 3, None, b, None, None) == -2
    assert sl(b, b, None, _lib.dims_arg((4, 4, 4)), 4, ctypes.byref(p), b, None, None) == -1
    assert b"which" in lib.msc_last_error_string()
    assert sl(b, b, None, _lib.dims_arg((2048, 2048, 1100)), 3, ctypes.byref(p), b, None, None) == -8


def test_cli_usage_message():
    exe = build.build_cli()
    res = subprocess.run([str(exe)], capture_output=True, text=True)
    assert res.returncode == 0
    assert "Usage: X Y Z filename per_x per_y per_z" in res.stdout


def test_ondemandaccurate_usage_message():
    build.build_cli()
    exe = build.BIN / "ondemandaccurate"
    for args in ([], ["64", "64", "64", "f.raw", "1e-4", "1e-6", "4000", "0", "0", "1", "1"]):  # 11: one short
        res = subprocess.run([str(exe), *args], capture_output=True, text=True)
        assert res.returncode == 0
        assert "Usage: X Y Z filename error_threshold grad_threshold maxnumiter" in res.stdout


def test_api_mesh_mirror():
    from msceer_gb300 import TopologicalRegularGrid3D, DiscreteGradientLabeling
    import numpy as np
    m = TopologicalRegularGrid3D(4, 3, 2)
    assert m.XYZ() == (7, 5, 3) and m.numCells() == 105
    ids = np.arange(m.numCells())
    c = m.cellid2Coords(ids)
    assert np.array_equal(m.coords2Cellid(c), ids)
    assert m.dimension(0) == 0 and m.dimension(1) == 1 and m.dimension(7 + 1) == 2
    assert m.boundaryValue(0) == 3 and m.boundaryValue(7 + 1) == 1 and m.boundaryValue(7 * 5 + 7 + 1) == 0
    g = DiscreteGradientLabeling(m)
    g.data[1] = 1 | (1 << 2)  # assigned, pair -x
    assert g.getPair(1) == 0 and g.getAssigned(1) == 1 and not g.getCritical(1)
