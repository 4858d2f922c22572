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


def load_ref():
    """The reference compiled from its own sources, or None where it is absent."""
    if not REF_SO.exists():
        return None
    lib = ctypes.CDLL(str(REF_SO))
    lib.ref_steepest_lstar_3d.argtypes = [_VP, ctypes.c_longlong, ctypes.c_longlong, ctypes.c_longlong,
                                          ctypes.c_int, ctypes.c_char_p, _VP]
    lib.ref_lstar_grad_2d.argtypes = [_VP, ctypes.c_longlong, ctypes.c_longlong, ctypes.c_int,
                                      ctypes.c_char_p, _VP]
    return lib


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
