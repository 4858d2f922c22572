"""The CUDA lower-star core, compiled for the host, against the oracle (no GPU).

tests/lstar_core_host.cpp drives msceer_gb300/csrc/lstar_core.cuh -- the exact
per-vertex code of the kernel -- over whole volumes; its bytes (pairs, flag and the
ascending-manifold roots) must equal the oracle's once the oracle's closure is run."""
import ctypes
import subprocess
from pathlib import Path

import numpy as np
import pytest

import oracle_lib
from msceer_gb300 import fields

HERE = Path(__file__).resolve().parent


@pytest.fixture(scope="module")
def core(tmp_path_factory):
    out = tmp_path_factory.mktemp("core") / "libcore.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-o", str(out),
                    str(HERE / "lstar_core_host.cpp")], check=True)
    lib = ctypes.CDLL(str(out))
    lib.core_pairs_3d.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64,
                                  ctypes.c_void_p, ctypes.c_uint32]
    lib.core_pairs_2d.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p, ctypes.c_uint32]
    lib.core_conform_3d.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p,
                                    ctypes.c_void_p, ctypes.c_uint32]
    return lib


def enc_map(dims):
    """The pair-code map of the library for these dims (first equal-stride axis)."""
    nd = len(dims)
    d = [2 * v - 1 for v in dims] + [1] * (3 - nd)
    cs = [1, d[0], d[0] * d[1]]
    m = 0
    for c in range(6):
        a, s = c >> 1, c & 1
        e = c
        if nd == 3:
            for b in range(3):
                if cs[b] == cs[a]:
                    e = 2 * b + s
                    break
        m |= e << (3 * c)
    return m


def core_grad(core, f):
    f = np.ascontiguousarray(f, dtype=np.float32)
    dims = f.shape[::-1]
    g = np.zeros(int(np.prod([2 * v - 1 for v in dims])), dtype=np.uint8)
    if f.ndim == 3:
        core.core_pairs_3d(f.ctypes.data, *dims, g.ctypes.data, enc_map(dims))
    else:
        core.core_pairs_2d(f.ctypes.data, *dims, g.ctypes.data, enc_map(dims))
    return g


def check(core, oracle, f):
    dims = f.shape[::-1]
    got = core_grad(core, f)
    want = oracle.grad(f)
    assert np.array_equal(got & 0x1F, want & 0x1F), oracle_lib.describe_mismatch(got & 0x1F, want & 0x1F, dims)
    # roots of the closure as the kernel writes them
    d = [2 * v - 1 for v in dims]
    ids = np.arange(got.size)
    c = [ids % d[0], (ids // d[0]) % d[1]] + ([ids // (d[0] * d[1])] if len(dims) == 3 else [])
    dim = sum(ci & 1 for ci in c)
    crit = ((want >> 2) & 7) == 7
    root = np.full(got.size, 3)
    root[crit & (dim == 1)] = 2
    root[crit & (dim == 2)] = 1
    root[crit & (dim == 3)] = 0
    assert np.array_equal(got >> 5, root)
    assert np.array_equal(oracle.ldir(got, dims), want)


@pytest.mark.parametrize("case", oracle_lib.load_golden_small(), ids=lambda c: c[0])
def test_core_golden(core, oracle, case):
    check(core, oracle, case[1])


@pytest.mark.parametrize("shape", [(31, 17, 9), (40, 37, 1), (1, 20, 23), (48, 48, 48)])
@pytest.mark.parametrize("kind", ["k3", "quant3", "gauss"])
def test_core_random(core, oracle, shape, kind):
    if kind == "gauss":
        f = fields.gaussian_sum(shape, 8, seed=3)
    else:
        f = fields.power_law_field(shape, seed=5)
        if kind == "quant3":
            f = fields.quantized(f, 3)
    check(core, oracle, f)


def test_core_2d(core, oracle):
    for shape in [(300, 211), (1, 40), (40, 1)]:
        f = fields.quantized(fields.power_law_field(shape, seed=2), 4)
        check(core, oracle, f)


@pytest.mark.parametrize("shape", [(40, 36, 32), (31, 17, 9), (33, 2, 20)])
def test_core_conform(core, oracle, shape):
    """The conforming re-pairing of the kernel core against the oracle: the restriction
    labels of the oracle's own final labels, the recomputed lower stars, then the
    closure and flag of both must give the same bytes."""
    f = fields.gaussian_sum(shape, 8, seed=5)
    gt = 1e-6 * float(np.abs(f).max())
    base = oracle.grad(f)
    lab = oracle.labels(f, base, 1e-4, gt, 4000, 0.25, 0.0)
    restrict = oracle.boundary_labels(f, lab["asc"], lab["dsc"])
    assert (restrict > 0).any()
    want = oracle.conform(f, restrict, base)
    dims = f.shape[::-1]
    got = base.copy()
    n = core.core_conform_3d(np.ascontiguousarray(f).ctypes.data, *dims, restrict.ctypes.data, got.ctypes.data,
                             enc_map(dims))
    assert n > 0
    # the recomputed cells carry closure roots: run the closure (and the flag) as the library does
    d = [2 * v - 1 for v in dims]
    ids = np.arange(got.size)
    dim = sum(ci & 1 for ci in (ids % d[0], (ids // d[0]) % d[1], ids // (d[0] * d[1])))
    crit = ((got >> 2) & 7) == 7
    root = np.full(got.size, 3, dtype=np.uint8)
    root[crit & (dim == 1)] = 2
    root[crit & (dim == 2)] = 1
    root[crit & (dim == 3)] = 0
    got = (got & 0x1F) | (root << 5)
    assert np.array_equal(oracle.ldir(got, dims), want), oracle_lib.describe_mismatch(oracle.ldir(got, dims), want,
                                                                                       dims)
