"""Parity of the CUDA .grad path (through the C ABI) with the oracle and with the
reference's golden outputs.  Bit-exact: every byte must match."""
import hashlib
import json
import os
import subprocess
from pathlib import Path

import numpy as np
import pytest

import oracle_lib
from msceer_gb300 import fields

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"


def dev_grad(f, device):
    import torch
    from msceer_gb300 import lower_star_grad
    t = torch.from_numpy(np.ascontiguousarray(f)).to(device)
    g = lower_star_grad(t)
    torch.cuda.synchronize()
    return g.cpu().numpy()


@pytest.mark.parametrize("case", oracle_lib.load_golden_small(), ids=lambda c: c[0])
def test_golden_small_device_path(gpu, case):
    name, f, want = case
    got = dev_grad(f, gpu)
    assert np.array_equal(got, want), oracle_lib.describe_mismatch(got, want, f.shape[::-1])


@pytest.mark.parametrize("case", oracle_lib.load_golden_small()[::5], ids=lambda c: c[0])
def test_golden_small_host_path(gpu, case):
    from msceer_gb300 import lower_star_grad
    name, f, want = case
    got = lower_star_grad(f)
    assert np.array_equal(got, want), oracle_lib.describe_mismatch(got, want, f.shape[::-1])


@pytest.mark.parametrize("key", ["gauss16_64", "k3_96x80x72", "k3_2d_512x384"])
def test_golden_large(gpu, oracle, key):
    spec = json.loads((GOLDEN / "grad_large.json").read_text())[key]
    f = eval("fields." + spec["generator"], {"fields": fields})
    got = dev_grad(f, gpu)
    if hashlib.sha256(f.tobytes()).hexdigest() == spec["f_sha256"]:
        assert hashlib.sha256(got.tobytes()).hexdigest() == spec["sha256"]
    want = oracle.grad(f)
    assert np.array_equal(got, want), oracle_lib.describe_mismatch(got, want, f.shape[::-1])


SHAPES_3D = [(2, 2, 2), (3, 3, 3), (31, 17, 9), (33, 16, 17), (65, 7, 40), (100, 37, 3), (1, 40, 37),
             (40, 1, 37), (40, 37, 1), (129, 63, 35)]


@pytest.mark.parametrize("shape", SHAPES_3D)
@pytest.mark.parametrize("kind", ["k3", "quant3", "gauss"])
def test_random_shapes_vs_oracle(gpu, oracle, shape, kind):
    if kind == "gauss":
        f = fields.gaussian_sum(shape, 8, seed=sum(shape))
    else:
        f = fields.power_law_field(shape, seed=sum(shape))
        if kind == "quant3":
            f = fields.quantized(f, 3)
    got = dev_grad(f, gpu)
    want = oracle.grad(f)
    assert np.array_equal(got, want), oracle_lib.describe_mismatch(got, want, shape)


@pytest.mark.parametrize("shape", [(2, 2), (3, 5), (257, 129), (1000, 77), (64, 300), (1, 50), (50, 1)])
@pytest.mark.parametrize("kind", ["k3", "quant2"])
def test_random_shapes_2d_vs_oracle(gpu, oracle, shape, kind):
    f = fields.power_law_field(shape, seed=7)
    if kind == "quant2":
        f = fields.quantized(f, 2)
    got = dev_grad(f, gpu)
    want = oracle.grad(f)
    assert np.array_equal(got, want), oracle_lib.describe_mismatch(got, want, shape)


def test_constant_field_all_ties(gpu, oracle):
    f = np.zeros((20, 21, 22), dtype=np.float32)
    assert np.array_equal(dev_grad(f, gpu), oracle.grad(f))
    f = np.full((33, 40), -0.0, dtype=np.float32)
    f[::3] = 0.0
    assert np.array_equal(dev_grad(f, gpu), oracle.grad(f))


def test_stages_compose(gpu, oracle):
    import torch
    from msceer_gb300 import ascending_manifold_dims, lower_star_grad, lower_star_pairs
    f = fields.power_law_field((70, 50, 44), seed=9)
    t = torch.from_numpy(f).to(gpu)
    g = lower_star_pairs(t)
    p = g.cpu().numpy()
    want = oracle.grad(f)
    assert np.array_equal(p & 0x1F, want & 0x1F)          # assigned, flag, pair
    passes = ascending_manifold_dims(g, f.shape[::-1])
    assert passes >= 1
    assert np.array_equal(g.cpu().numpy(), want)
    assert np.array_equal(lower_star_grad(t).cpu().numpy(), want)


def test_nan_input_rejected(gpu):
    import torch
    from msceer_gb300 import _lib, lower_star_grad
    f = np.zeros((8, 8, 8), dtype=np.float32)
    f[3, 4, 5] = np.nan
    with pytest.raises(_lib.MscError) as e:
        lower_star_grad(torch.from_numpy(f).to(gpu))
    assert e.value.code == -5


def test_cli_drop_in(gpu, oracle, tmp_path):
    from msceer_gb300 import build
    exe = build.build_cli()
    f = fields.gaussian_sum((24, 20, 16), 6, seed=4)
    raw = tmp_path / "vol.raw"
    f.tofile(raw)
    res = subprocess.run([str(exe), "24", "20", "16", str(raw), "0", "0", "0", "8"], capture_output=True, text=True)
    assert res.returncode == 1, res.stderr  # the reference's exit status after a run
    got = np.fromfile(str(raw) + ".grad", dtype=np.uint8)
    assert np.array_equal(got, oracle.grad(f))
    assert (tmp_path / "vol.raw.steep.gtime.txt").read_text().startswith("Total Overall 0 ")


def test_256_cubed_vs_oracle(gpu, oracle):
    f = fields.power_law_field((256, 256, 256), seed=1)
    got = dev_grad(f, gpu)
    want = oracle.grad(f, nthreads=os.cpu_count() or 4)
    assert np.array_equal(got, want), oracle_lib.describe_mismatch(got, want, (256, 256, 256))


def _properties(g, dims, chunk=1 << 26):
    """Size-independent invariants of a discrete gradient .grad, checked in chunks
    so the full-size volumes stay within a few GB of scratch."""
    import torch
    nd = len(dims)
    d = [2 * x - 1 for x in dims]
    strides = [1, d[0], d[0] * d[1]][:nd]
    offs = torch.tensor([s * sg for s in strides for sg in (1, -1)] + [0] * (8 - 2 * nd), device=g.device)
    cnt = [0] * (nd + 1)
    n = g.numel()
    for lo in range(0, n, chunk):
        hi = min(n, lo + chunk)
        ids = torch.arange(lo, hi, device=g.device, dtype=torch.int64)
        c = [ids % d[0], (ids // d[0]) % d[1]] + ([ids // (d[0] * d[1])] if nd == 3 else [])
        dim = sum((ci & 1) for ci in c)
        gi = g[lo:hi].to(torch.int32)
        assert bool((gi & 1).all()), "unassigned cell"
        code = (gi >> 2) & 7
        crit = code == 7
        for k in range(nd + 1):
            cnt[k] += int((crit & (dim == k)).sum())
        nc = ~crit
        partner = ids[nc] + offs[code[nc].long()]
        assert bool(((partner >= 0) & (partner < n)).all())
        pcode = (g[partner].to(torch.int32) >> 2) & 7
        assert bool((pcode != 7).all())
        assert bool((partner + offs[pcode.long()] == ids[nc]).all()), "pairing not symmetric"
        pc = [partner % d[0], (partner // d[0]) % d[1]] + ([partner // (d[0] * d[1])] if nd == 3 else [])
        pdim = sum((ci & 1) for ci in pc)
        assert bool(((pdim - dim[nc]).abs() == 1).all())
        flag = (gi >> 1) & 1
        bnd = sum(((ci == 0) | (ci == di - 1)).to(torch.int32) for ci, di in zip(c, d))
        assert bool((flag == (bnd > 0).to(torch.int32)).all())
    euler = sum((-1) ** k * v for k, v in enumerate(cnt))
    assert euler == 1, cnt                       # alternating sum of critical cells = chi(box)
    return cnt


def _vs_reference_and_oracle(gpu, oracle, key, shape):
    """The .grad scale workload byte for byte: against the reference's own output (by
    hash, where this platform regenerates the fixture's input bit for bit) and against
    the multi-threaded oracle (always)."""
    import torch
    from msceer_gb300 import lower_star_grad
    spec = json.loads((GOLDEN / "grad_large.json").read_text())[key]
    f = eval("fields." + spec["generator"], {"fields": fields})
    t = torch.from_numpy(f).to(gpu)
    g = lower_star_grad(t)
    assert torch.equal(g, lower_star_grad(t))    # deterministic run to run
    got = g.cpu().numpy()
    del g, t
    if hashlib.sha256(f.tobytes()).hexdigest() == spec["f_sha256"]:
        assert hashlib.sha256(got.tobytes()).hexdigest() == spec["sha256"]
    want = oracle.grad(f)
    assert np.array_equal(got, want), oracle_lib.describe_mismatch(got, want, shape)
    cnt = _properties(torch.from_numpy(got).to(gpu), shape)
    assert cnt[0] > 0 and cnt[-1] > 0


def test_512_cubed_vs_reference(gpu, oracle):
    _vs_reference_and_oracle(gpu, oracle, "k3_512cubed", (512, 512, 512))


def test_8192_squared_vs_reference(gpu, oracle):
    _vs_reference_and_oracle(gpu, oracle, "k3_8192sq", (8192, 8192))


@pytest.mark.parametrize("shape", [(96, 80, 72), (700, 900)], ids=["3d", "2d"])
def test_frontier_overflow_falls_back_to_passes(gpu, oracle, monkeypatch, shape):
    """A frontier queue too small for the cross-tile walks hands the closure to the
    multi-pass form, which finishes it from the intermediate state."""
    monkeypatch.setenv("MSC_LDIR_QUEUE_CAP", "8")
    from msceer_gb300 import _lib
    f = fields.power_law_field(shape, seed=12)
    got = dev_grad(f, gpu)
    assert _lib.load().msc_last_ldir_passes() >= 3  # tile + check + at least one full tile pass
    assert np.array_equal(got, oracle.grad(f))


def test_ascending_manifold_dims_idempotent(gpu, oracle):
    import torch
    from msceer_gb300 import ascending_manifold_dims
    f = fields.power_law_field((64, 72, 80), seed=13)
    want = oracle.grad(f)
    g = torch.from_numpy(want.copy()).to(gpu)
    ascending_manifold_dims(g, f.shape[::-1])
    assert np.array_equal(g.cpu().numpy(), want)


def test_batch_of_uneven_volumes_equals_single_calls(gpu):
    """msc_lower_star_grad_batch_3d: volumes of different shapes in shared launches give
    the same bytes as one call per volume."""
    import torch
    from msceer_gb300 import lower_star_grad, lower_star_grad_batch
    rng = np.random.default_rng(21)
    shapes = [tuple(int(v) for v in rng.integers(3, 70, size=3)) for _ in range(9)] + [(2, 2, 2), (1, 5, 7)]
    vols = [torch.from_numpy(fields.power_law_field(s, seed=i)).to(gpu) for i, s in enumerate(shapes)]
    got = lower_star_grad_batch(vols)
    for v, g in zip(vols, got):
        assert torch.equal(g, lower_star_grad(v))


def test_batch_of_48_volumes(gpu):
    """Volume indices of 32 and above (the frontier entries carry the index in their top bits)."""
    import torch
    from msceer_gb300 import lower_star_grad, lower_star_grad_batch
    rng = np.random.default_rng(22)
    shapes = [tuple(int(v) for v in rng.integers(16, 48, size=3)) for _ in range(48)]
    vols = [torch.from_numpy(fields.power_law_field(s, seed=100 + i)).to(gpu) for i, s in enumerate(shapes)]
    got = lower_star_grad_batch(vols)
    for v, g in zip(vols, got):
        assert torch.equal(g, lower_star_grad(v))


def test_batch_graph_replay_sees_new_values(gpu):
    """The batch graph is kept while the same buffers come back: a replay after the
    volumes changed in place gives the .grad of the new values."""
    import torch
    from msceer_gb300 import lower_star_grad, lower_star_grad_batch
    shapes = [(40, 36, 33), (17, 64, 50), (64, 64, 64), (5, 9, 70)]
    vols = [torch.from_numpy(fields.power_law_field(s, seed=200 + i)).to(gpu) for i, s in enumerate(shapes)]
    outs = lower_star_grad_batch(vols)
    for v, g in zip(vols, outs):
        assert torch.equal(g, lower_star_grad(v))
    for v in vols:
        v.mul_(-1.0)
    again = lower_star_grad_batch(vols, outs)
    for v, g in zip(vols, again):
        assert torch.equal(g, lower_star_grad(v))


def test_batch_graph_overflow_falls_back_to_passes(gpu, oracle, monkeypatch):
    monkeypatch.setenv("MSC_LDIR_QUEUE_CAP", "8")
    import torch
    from msceer_gb300 import lower_star_grad_batch
    fs = [fields.power_law_field(s, seed=300 + i) for i, s in enumerate([(70, 66, 60), (33, 80, 41)])]
    got = lower_star_grad_batch([torch.from_numpy(f).to(gpu) for f in fs])
    for f, g in zip(fs, got):
        assert np.array_equal(g.cpu().numpy(), oracle.grad(f))
