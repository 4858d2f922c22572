"""The allocation-free ldir entry point (msc_ascending_manifold_dims_3d_static).

It serves applications that own all device memory through their own pool and do not
allow a library to call cudaMalloc; its pass scratch lives in a fixed array in the
library.  Through the C ABI, calls in a row must give exactly (bit for bit) what the
allocating entry point gives -- also after a larger call has left its flags in the
shared array, near the array's tile limit and with a single-vertex axis.  This file
sorts last so that a run that stops at the first failure has run every other test
already."""
import ctypes

import numpy as np
import pytest

from msceer_gb300 import _lib, fields

pytestmark = pytest.mark.gpu


def compare_entries(gpu, f, calls=2):
    import torch
    from msceer_gb300 import lower_star_pairs

    lib = _lib.load()
    dims = _lib.dims_arg(f.shape[::-1])
    stage1 = lower_star_pairs(torch.from_numpy(f).to(gpu))
    stream = ctypes.c_void_p(torch.cuda.current_stream(gpu).cuda_stream)
    want = stage1.clone()
    passes = ctypes.c_int(0)
    _lib.check(lib.msc_ascending_manifold_dims_3d(ctypes.c_void_p(want.data_ptr()), dims, stream,
                                                  ctypes.byref(passes)), "msc_ascending_manifold_dims_3d")
    for call in range(calls):
        got = stage1.clone()
        p2 = ctypes.c_int(0)
        rc = lib.msc_ascending_manifold_dims_3d_static(ctypes.c_void_p(got.data_ptr()), dims, stream, ctypes.byref(p2))
        _lib.check(rc, "msc_ascending_manifold_dims_3d_static")
        torch.cuda.synchronize(gpu)
        assert torch.equal(got, want), f"call {call}: {int((got != want).sum())} bytes differ"
        assert p2.value >= 1  # tile passes of the multi-pass form
    del stage1, want


def test_static_scratch_entry_matches_allocating_entry(gpu):
    compare_entries(gpu, fields.power_law_field((70, 50, 44), seed=9))


def test_static_scratch_entry_after_a_larger_call(gpu):
    """Flags a larger call leaves in the shared array do not leak into a smaller one."""
    compare_entries(gpu, fields.power_law_field((200, 180, 150), seed=11), calls=1)
    compare_entries(gpu, fields.power_law_field((60, 40, 30), seed=12))


def test_static_scratch_entry_single_vertex_axis(gpu):
    compare_entries(gpu, fields.power_law_field((1, 40, 37), seed=13))


def test_static_scratch_entry_near_its_tile_limit(gpu):
    """960^3 vertices: 432,000 of the 524,288 tiles the array holds (white noise: any
    field serves the closure, and it is quick to make)."""
    f = np.random.default_rng(14).standard_normal((960, 960, 960), dtype=np.float32)
    compare_entries(gpu, f, calls=1)


def test_static_scratch_entry_rejects_oversized_volume(gpu):
    lib = _lib.load()
    buf = ctypes.create_string_buffer(16)
    rc = lib.msc_ascending_manifold_dims_3d_static(ctypes.c_void_p(ctypes.addressof(buf)),
                                                   _lib.dims_arg((2048, 2048, 2048)), None, None)
    assert rc == -8
    assert b"static scratch" in lib.msc_last_error_string()
