"""ctypes access to the test-only checkers under oracle/ (built by
`make -C oracle`; the reference harness only where the reference sources exist)."""
from __future__ import annotations

import ctypes
import os
import subprocess
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
ORACLE_SO = ROOT / "oracle" / "_build" / "libmsc_oracle.so"
REF_SO = ROOT / "oracle" / "_ref" / "libmsc_ref.so"

_I64 = ctypes.c_int64
_VP = ctypes.c_void_p


class LabelParams(ctypes.Structure):
    """oracle_label_params (oracle/msc_oracle.h)."""
    _fields_ = [("error_threshold", ctypes.c_float), ("gradient_threshold", ctypes.c_float),
                ("iteration_limit", ctypes.c_int), ("max_step", ctypes.c_double),
                ("presimp_threshold", ctypes.c_float)]


STAGES = ("asc_terminal", "asc_integrated", "dsc_terminal", "dsc_integrated")


class Oracle:
    def __init__(self, lib):
        self.lib = lib
        for n in ("oracle_grad_3d", "oracle_lstar_pairs_3d"):
            getattr(lib, n).argtypes = [_VP, _I64, _I64, _I64, _VP, ctypes.c_int]
        for n in ("oracle_grad_2d", "oracle_lstar_pairs_2d"):
            getattr(lib, n).argtypes = [_VP, _I64, _I64, _VP, ctypes.c_int]
        lib.oracle_ldir_3d.argtypes = [_I64, _I64, _I64, _VP]
        lib.oracle_ldir_2d.argtypes = [_I64, _I64, _VP]
        lib.oracle_flag_3d.argtypes = [_I64, _I64, _I64, _VP]
        lib.oracle_flag_2d.argtypes = [_I64, _I64, _VP]
        lib.oracle_central_diff_3d.argtypes = [_VP, _I64, _I64, _I64, _VP]
        lib.oracle_central_diff_2d.argtypes = [_VP, _I64, _I64, _VP]
        lib.oracle_labels_3d.argtypes = [_VP, _VP, _I64, _I64, _I64, ctypes.c_int, ctypes.POINTER(LabelParams),
                                         _VP, _VP, _VP]
        lib.oracle_terminal_regions_3d.argtypes = [_VP, _VP, _I64, _I64, _I64, ctypes.c_int, ctypes.c_float, _VP]
        lib.oracle_clean_regions_3d.argtypes = [_VP, _I64, _I64, _I64, ctypes.c_int, _VP]
        lib.oracle_boundary_labels_3d.argtypes = [_VP, _I64, _I64, _I64, _VP, _VP, _VP]
        lib.oracle_conform_3d.argtypes = [_VP, _I64, _I64, _I64, _VP, _VP, ctypes.c_int]
        lib.oracle_ms_graph_3d.argtypes = [_VP, _VP, _I64, _I64, _I64, _VP, _I64, _VP, _VP, _VP, _VP, _I64, _VP, _VP,
                                           _VP, _VP]
        lib.oracle_saddle_lines_3d.argtypes = [_VP, _VP, _I64, _I64, _I64, ctypes.c_int, ctypes.POINTER(LabelParams),
                                               _VP]
        lib.oracle_saddle_lines_zeroed_3d.argtypes = [_VP, _VP, _VP, _I64, _I64, _I64, ctypes.c_int,
                                                      ctypes.POINTER(LabelParams), _VP]
        lib.oracle_ondemand_grad_3d.argtypes = [_VP, _VP, _I64, _I64, _I64, ctypes.POINTER(LabelParams),
                                                ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, _VP, _VP]

    def ondemand_grad(self, f, grad, flags, error_threshold, gradient_threshold, iteration_limit, max_step,
                      presimp=0.0):
        """ondemandaccurate's accurate .grad for flags (needASC1, needDSC1, needASC2,
        needDSC2) at one thread: (restriction labels, .grad)."""
        f = np.ascontiguousarray(f, dtype=np.float32)
        grad = np.ascontiguousarray(grad, dtype=np.uint8)
        restrict = np.empty(grad.size, np.uint8)
        out = np.empty(grad.size, np.uint8)
        p = LabelParams(error_threshold, gradient_threshold, iteration_limit, max_step, presimp)
        assert self.lib.oracle_ondemand_grad_3d(f.ctypes.data, grad.ctypes.data, *f.shape[::-1], ctypes.byref(p),
                                                *[int(x) for x in flags], restrict.ctypes.data, out.ctypes.data) == 0
        return restrict, out

    def saddle_lines(self, f, grad, which, error_threshold, gradient_threshold, iteration_limit, max_step,
                     cells=None, zeroed=None):
        """ondemandaccurate's saddle streamline digitizers (which: 1 ascending from the
        2-saddles, label 4; 2 descending from the 1-saddles, label 5; 3 both) at one
        thread, into a copy of `cells` (one byte per cell; zeros when not given); the
        gradient is zero at the vertices whose bit the uint32 bitmap `zeroed` sets."""
        f = np.ascontiguousarray(f, dtype=np.float32)
        grad = np.ascontiguousarray(grad, dtype=np.uint8)
        nc = int(np.prod([2 * d - 1 for d in f.shape]))
        out = np.zeros(nc, np.uint8) if cells is None else np.array(cells, dtype=np.uint8, copy=True)
        p = LabelParams(error_threshold, gradient_threshold, iteration_limit, max_step, 0.0)
        if zeroed is None:
            rc = self.lib.oracle_saddle_lines_3d(f.ctypes.data, grad.ctypes.data, *f.shape[::-1], which,
                                                 ctypes.byref(p), out.ctypes.data)
        else:
            zeroed = np.ascontiguousarray(zeroed, dtype=np.uint32)
            assert zeroed.size * 32 >= f.size
            rc = self.lib.oracle_saddle_lines_zeroed_3d(f.ctypes.data, grad.ctypes.data, zeroed.ctypes.data,
                                                        *f.shape[::-1], which, ctypes.byref(p), out.ctypes.data)
        assert rc == 0
        return out

    def labels(self, f, grad, error_threshold, gradient_threshold, iteration_limit, max_step, presimp):
        """ASC and DSC labels (regions named by their smallest seed vertex) plus stages."""
        f = np.ascontiguousarray(f, dtype=np.float32)
        n = f.size
        asc = np.empty(n, np.int32)
        dsc = np.empty(n, np.int32)
        st = np.empty(4 * n, np.int32)
        p = LabelParams(error_threshold, gradient_threshold, iteration_limit, max_step, presimp)
        rc = self.lib.oracle_labels_3d(f.ctypes.data, grad.ctypes.data, *f.shape[::-1], 3, ctypes.byref(p),
                                       asc.ctypes.data, dsc.ctypes.data, st.ctypes.data)
        assert rc == 0
        out = {"asc": asc, "dsc": dsc}
        for i, k in enumerate(STAGES):
            out[k] = st[i * n:(i + 1) * n]
        return out

    def clean(self, f, labels, direction):
        """IsolatedCCRegionRemoverNEW on a copy of `labels` (direction -1 ASC, +1 DSC)."""
        f = np.ascontiguousarray(f, dtype=np.float32)
        out = np.array(labels, dtype=np.int32, copy=True)
        assert self.lib.oracle_clean_regions_3d(f.ctypes.data, *f.shape[::-1], int(direction), out.ctypes.data) == 0
        return out

    def boundary_labels(self, f, asc, dsc):
        """VertexLabelingToBoundaryLabeling MIN (asc) then MAX (dsc) restriction labels."""
        f = np.ascontiguousarray(f, dtype=np.float32)
        n = int(np.prod([2 * d - 1 for d in f.shape]))
        out = np.empty(n, np.uint8)
        a = None if asc is None else np.ascontiguousarray(asc, dtype=np.int32)
        d = None if dsc is None else np.ascontiguousarray(dsc, dtype=np.int32)
        assert self.lib.oracle_boundary_labels_3d(f.ctypes.data, *f.shape[::-1], None if a is None else a.ctypes.data,
                                                  None if d is None else d.ctypes.data, out.ctypes.data) == 0
        return out

    def conform(self, f, restrict, base_grad, nthreads=0):
        """The accurate 3-manifold .grad from the base .grad and the restriction labels."""
        f = np.ascontiguousarray(f, dtype=np.float32)
        g = np.array(base_grad, dtype=np.uint8, copy=True)
        r = np.ascontiguousarray(restrict, dtype=np.uint8)
        assert self.lib.oracle_conform_3d(f.ctypes.data, *f.shape[::-1], r.ctypes.data, g.ctypes.data, nthreads) == 0
        return g

    def ms_graph(self, f, grad, build=(1, 0, 1)):
        """MorseSmaleComplexBasic::ComputeFromGrad (no arc geometry): a dict of node and arc arrays."""
        f = np.ascontiguousarray(f, dtype=np.float32)
        grad = np.ascontiguousarray(grad, dtype=np.uint8)
        b = (ctypes.c_int * 3)(*build)
        counts = np.zeros(2, np.int64)
        self.lib.oracle_ms_graph_3d(grad.ctypes.data, f.ctypes.data, *f.shape[::-1], b, 0, None, None, None, None, 0,
                                    None, None, None, counts.ctypes.data)
        return _ms_graph_call(lambda *a: self.lib.oracle_ms_graph_3d(grad.ctypes.data, f.ctypes.data, *f.shape[::-1],
                                                                     b, *a), counts)

    def central_diff(self, f: np.ndarray) -> np.ndarray:
        """(..., ND) float64 gradient, the reference's Vec3d array."""
        f = np.ascontiguousarray(f, dtype=np.float32)
        g = np.empty(f.shape + (f.ndim,), dtype=np.float64)
        if f.ndim == 3:
            assert self.lib.oracle_central_diff_3d(f.ctypes.data, *f.shape[::-1], g.ctypes.data) == 0
        else:
            assert self.lib.oracle_central_diff_2d(f.ctypes.data, *f.shape[::-1], g.ctypes.data) == 0
        return g

    def grad(self, f: np.ndarray, nthreads: int = 0) -> np.ndarray:
        f = np.ascontiguousarray(f, dtype=np.float32)
        dims = f.shape[::-1]
        n = int(np.prod([2 * d - 1 for d in dims]))
        g = np.empty(n, dtype=np.uint8)
        if f.ndim == 3:
            rc = self.lib.oracle_grad_3d(f.ctypes.data, *dims, g.ctypes.data, nthreads)
        else:
            rc = self.lib.oracle_grad_2d(f.ctypes.data, *dims, g.ctypes.data, nthreads)
        assert rc == 0
        return g

    def pairs(self, f: np.ndarray, nthreads: int = 0) -> np.ndarray:
        f = np.ascontiguousarray(f, dtype=np.float32)
        dims = f.shape[::-1]
        n = int(np.prod([2 * d - 1 for d in dims]))
        g = np.empty(n, dtype=np.uint8)
        fn = self.lib.oracle_lstar_pairs_3d if f.ndim == 3 else self.lib.oracle_lstar_pairs_2d
        assert fn(f.ctypes.data, *dims, g.ctypes.data, nthreads) == 0
        return g

    def ldir(self, g: np.ndarray, dims) -> np.ndarray:
        g = g.copy()
        fn = self.lib.oracle_ldir_3d if len(dims) == 3 else self.lib.oracle_ldir_2d
        assert fn(*dims, g.ctypes.data) == 0
        return g


def build() -> None:
    subprocess.run(["make", "-s", "-C", str(ROOT / "oracle")], check=True)


def load() -> Oracle:
    if not ORACLE_SO.exists() or ORACLE_SO.stat().st_mtime < (ROOT / "oracle" / "msc_oracle.c").stat().st_mtime:
        build()
    return Oracle(ctypes.CDLL(str(ORACLE_SO)))


def _ms_graph_call(fn, counts):
    nn, na = int(counts[0]), int(counts[1])
    out = {"node_cell": np.empty(nn, np.int64), "node_value": np.empty(nn, np.float32),
           "node_dim": np.empty(nn, np.uint8), "node_boundary": np.empty(nn, np.uint8),
           "arc_lower": np.empty(na, np.int32), "arc_upper": np.empty(na, np.int32),
           "arc_persistence": np.empty(na, np.float32)}
    c2 = np.zeros(2, np.int64)
    assert fn(nn, out["node_cell"].ctypes.data, out["node_value"].ctypes.data, out["node_dim"].ctypes.data,
              out["node_boundary"].ctypes.data, na, out["arc_lower"].ctypes.data, out["arc_upper"].ctypes.data,
              out["arc_persistence"].ctypes.data, c2.ctypes.data) == 0
    assert tuple(c2) == (nn, na)
    return out


def ref_ms_graph(lib, f, grad, build=(1, 0, 1), nthreads=1):
    """The reference's MorseSmaleComplexBasic::ComputeFromGrad on a .grad (extractmsc's
    setup), as ms_graph returns it."""
    f = np.ascontiguousarray(f, dtype=np.float32)
    grad = np.ascontiguousarray(grad, dtype=np.uint8)
    b = (ctypes.c_int * 3)(*build)
    counts = np.zeros(2, np.int64)
    dims = f.shape[::-1]
    lib.ref_ms_graph_3d(f.ctypes.data, *dims, grad.ctypes.data, b, nthreads, 0, None, None, None, None, 0, None, None,
                        None, counts.ctypes.data)
    return _ms_graph_call(lambda *a: lib.ref_ms_graph_3d(f.ctypes.data, *dims, grad.ctypes.data, b, nthreads, *a),
                          counts)


def load_ref():
    """The reference compiled from its own sources, or None where it is absent."""
    if not REF_SO.exists():
        return None
    lib = ctypes.CDLL(str(REF_SO))
    lib.ref_steepest_lstar_3d.argtypes = [_VP, ctypes.c_longlong, ctypes.c_longlong, ctypes.c_longlong,
                                          ctypes.c_int, ctypes.c_char_p, _VP]
    lib.ref_lstar_grad_2d.argtypes = [_VP, ctypes.c_longlong, ctypes.c_longlong, ctypes.c_int,
                                      ctypes.c_char_p, _VP]
    lib.ref_central_diff_3d.argtypes = [_VP, ctypes.c_longlong, ctypes.c_longlong, ctypes.c_longlong, _VP]
    lib.ref_ms_graph_3d.argtypes = [_VP, ctypes.c_longlong, ctypes.c_longlong, ctypes.c_longlong, _VP, _VP,
                                    ctypes.c_int, ctypes.c_longlong, _VP, _VP, _VP, _VP, ctypes.c_longlong, _VP, _VP,
                                    _VP, _VP]
    lib.ref_labels_3d.argtypes = [_VP, ctypes.c_longlong, ctypes.c_longlong, ctypes.c_longlong, ctypes.c_float,
                                  ctypes.c_float, ctypes.c_int, ctypes.c_float, _VP, _VP, _VP]
    lib.ref_ondemand_3d.argtypes = [_VP, ctypes.c_longlong, ctypes.c_longlong, ctypes.c_longlong, ctypes.c_float,
                                    ctypes.c_float, ctypes.c_int, ctypes.c_float, _VP, _VP, _VP, ctypes.c_int,
                                    ctypes.c_char_p, _VP]
    if hasattr(lib, "ref_ondemand_modes_3d"):
        lib.ref_ondemand_modes_3d.argtypes = [_VP, ctypes.c_longlong, ctypes.c_longlong, ctypes.c_longlong,
                                              ctypes.c_float, ctypes.c_float, ctypes.c_int, ctypes.c_float,
                                              ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_char_p,
                                              _VP]
    if hasattr(lib, "ref_saddle_lines_3d"):
        lib.ref_saddle_lines_3d.argtypes = [_VP, ctypes.c_longlong, ctypes.c_longlong, ctypes.c_longlong,
                                            ctypes.c_int, ctypes.c_float, ctypes.c_float, ctypes.c_int, _VP]
    return lib


def ref_ondemand_modes(lib, f, flags, error_threshold, gradient_threshold, iteration_limit, presimp=0.0):
    """The reference's ondemandaccurate for flags (needASC1, needDSC1, needASC2,
    needDSC2) at one thread: (restriction labels, the .grad it writes)."""
    f = np.ascontiguousarray(f, dtype=np.float32)
    nc = int(np.prod([2 * d - 1 for d in f.shape]))
    restrict = np.empty(nc, np.uint8)
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "o.grad").encode()
        assert lib.ref_ondemand_modes_3d(f.ctypes.data, *f.shape[::-1], error_threshold, gradient_threshold,
                                         iteration_limit, presimp, *[int(x) for x in flags], path,
                                         restrict.ctypes.data) == 0
        grad = np.fromfile(path.decode(), dtype=np.uint8)
    return restrict, grad


def ref_saddle_lines(lib, f, which, error_threshold, gradient_threshold, iteration_limit, cells=None):
    """The reference's saddle streamline digitizers at one thread (built with
    MAX_STEP_IN_GRID_CELLS = 0.25), as Oracle.saddle_lines returns them."""
    f = np.ascontiguousarray(f, dtype=np.float32)
    nc = int(np.prod([2 * d - 1 for d in f.shape]))
    out = np.zeros(nc, np.uint8) if cells is None else np.array(cells, dtype=np.uint8, copy=True)
    assert lib.ref_saddle_lines_3d(f.ctypes.data, *f.shape[::-1], which, error_threshold, gradient_threshold,
                                   iteration_limit, out.ctypes.data) == 0
    return out


def ref_labels(lib, f, error_threshold, gradient_threshold, iteration_limit, presimp):
    """The reference's ondemandaccurate ASC/DSC labels at one thread (built with
    MAX_STEP_IN_GRID_CELLS = 0.25), regions named by their smallest seed vertex."""
    f = np.ascontiguousarray(f, dtype=np.float32)
    n = f.size
    asc = np.empty(n, np.int32)
    dsc = np.empty(n, np.int32)
    st = np.empty(4 * n, np.int32)
    assert lib.ref_labels_3d(f.ctypes.data, *f.shape[::-1], error_threshold, gradient_threshold, iteration_limit,
                             presimp, asc.ctypes.data, dsc.ctypes.data, st.ctypes.data) == 0
    out = {"asc": asc, "dsc": dsc}
    for i, k in enumerate(STAGES):
        out[k] = st[i * n:(i + 1) * n]
    return out


def ref_ondemand(lib, f, error_threshold, gradient_threshold, iteration_limit, presimp):
    """ondemandaccurate with needASC2 = needDSC2 = 1 at one thread: the final ASC / DSC
    labels, the restriction labels and the accurate .grad it writes."""
    f = np.ascontiguousarray(f, dtype=np.float32)
    n = f.size
    nc = int(np.prod([2 * d - 1 for d in f.shape]))
    asc = np.empty(n, np.int32)
    dsc = np.empty(n, np.int32)
    restrict = np.empty(nc, np.uint8)
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "o.grad").encode()
        assert lib.ref_ondemand_3d(f.ctypes.data, *f.shape[::-1], error_threshold, gradient_threshold,
                                   iteration_limit, presimp, asc.ctypes.data, dsc.ctypes.data, None, 1, path,
                                   restrict.ctypes.data) == 0
        grad = np.fromfile(path.decode(), dtype=np.uint8)
    return {"asc": asc, "dsc": dsc, "restrict": restrict, "grad": grad}


def ref_grad(lib, f: np.ndarray, nthreads: int = 4) -> np.ndarray:
    f = np.ascontiguousarray(f, dtype=np.float32)
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "o.grad").encode()
        if f.ndim == 3:
            Z, Y, X = f.shape
            assert lib.ref_steepest_lstar_3d(f.ctypes.data, X, Y, Z, nthreads, path, None) == 0
        else:
            Y, X = f.shape
            assert lib.ref_lstar_grad_2d(f.ctypes.data, X, Y, max(1, min(nthreads, Y)), path, None) == 0
        return np.fromfile(path.decode(), dtype=np.uint8)


def load_golden_small():
    z = np.load(ROOT / "tests" / "golden" / "grad_small.npz")
    names = sorted({k.rsplit("__", 1)[0] for k in z.files})
    return [(n, z[f"{n}__f"], z[f"{n}__grad"]) for n in names]


def describe_mismatch(a: np.ndarray, b: np.ndarray, dims) -> str:
    if a.shape != b.shape:
        return f"size {a.size} != {b.size}"
    d = np.nonzero(a != b)[0]
    if d.size == 0:
        return "equal"
    dd = [2 * x - 1 for x in dims]
    out = [f"{d.size} cells differ"]
    for i in d[:6]:
        c = (i % dd[0], (i // dd[0]) % dd[1], i // (dd[0] * dd[1]))
        out.append(f"cell {i} {c}: got {a[i]:08b} want {b[i]:08b}")
    return "; ".join(out)
