"""Central-difference gradient kernel (through the C ABI) against the oracle:
bit-exact in f64, within half an ulp of the f64 value in f32."""
import ctypes

import numpy as np
import pytest

from msceer_gb300 import _lib, fields

pytestmark = pytest.mark.gpu


def run(f, device, layout):
    import torch
    lib = _lib.load()
    t = torch.from_numpy(np.ascontiguousarray(f)).to(device)
    nd = f.ndim
    dims = _lib.dims_arg(f.shape[::-1])
    stream = ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)
    if layout == "f64":
        out = torch.empty(f.shape + (nd,), dtype=torch.float64, device=device)
        fn = lib.msc_central_diff_grad_3d_f64 if nd == 3 else lib.msc_central_diff_grad_2d_f64
        rc = fn(ctypes.c_void_p(t.data_ptr()), dims, ctypes.c_void_p(out.data_ptr()), stream)
    else:
        width = nd if layout == 0 else (4 if nd == 3 else 2)
        out = torch.empty(f.shape + (width,), dtype=torch.float32, device=device)
        fn = lib.msc_central_diff_grad_3d if nd == 3 else lib.msc_central_diff_grad_2d
        rc = fn(ctypes.c_void_p(t.data_ptr()), dims, ctypes.c_void_p(out.data_ptr()), layout, stream)
    _lib.check(rc, "central_diff")
    torch.cuda.synchronize(device)
    return out.cpu().numpy()


@pytest.mark.parametrize("shape", [(2, 2, 2), (37, 21, 13), (128, 96, 64), (1, 9, 9), (300, 201)])
def test_gradient_f64_bit_exact(gpu, oracle, shape):
    f = fields.power_law_field(shape, seed=3)
    want = oracle.central_diff(f)
    got = run(f, gpu, "f64")
    assert np.array_equal(got.view(np.uint64), want.view(np.uint64))


@pytest.mark.parametrize("shape", [(37, 21, 13), (256, 128, 64), (300, 201)])
@pytest.mark.parametrize("layout", [0, 1])
def test_gradient_f32_half_ulp(gpu, oracle, shape, layout):
    f = fields.gaussian_sum(shape, 10, seed=2)
    want = oracle.central_diff(f)
    got = run(f, gpu, layout)[..., : f.ndim].astype(np.float64)
    # tolerance: the f32 result is the f64 value rounded once -> |err| <= ulp/2
    ulp = np.spacing(np.abs(want).astype(np.float32)).astype(np.float64)
    assert (np.abs(got - want) <= 0.5 * ulp).all()
    if layout == 1 and f.ndim == 3:
        assert (run(f, gpu, 1)[..., 3] == 0).all()
