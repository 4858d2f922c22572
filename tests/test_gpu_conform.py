"""ondemandaccurate's accurate 3-manifold .grad on the GPU (msc_conforming_grad_3d)
against the oracle, whose restriction labels and re-pairing equal the reference's byte
for byte (tests/test_oracle.py::test_conforming_grad_oracle_against_reference).

Given the same final labels the .grad is exact; end to end the GPU's own labels differ
from the oracle's on a small fraction of vertices (tests/test_gpu_labels.py), and the
.grad differs only in the lower stars next to those."""
import numpy as np
import pytest

import oracle_lib
from msceer_gb300 import fields

pytestmark = pytest.mark.gpu

FIELDS = {
    "gauss40": lambda: fields.gaussian_sum((40, 36, 32), 8, seed=5),
    "k3_32": lambda: fields.power_law_field((32, 30, 28), seed=6),
    "gauss64_cfg0": lambda: fields.gaussian_sum((64, 64, 64), 16, seed=0),
}


def oracle_side(oracle, f):
    gt = 1e-6 * float(np.abs(f).max())
    base = oracle.grad(f)
    lab = oracle.labels(f, base, 1e-4, gt, 4000, 0.25, 0.0)
    restrict = oracle.boundary_labels(f, lab["asc"], lab["dsc"])
    return base, lab, restrict, oracle.conform(f, restrict, base)


@pytest.mark.parametrize("name", list(FIELDS))
def test_conforming_grad_given_the_oracle_labels(gpu, oracle, name):
    import torch
    from msceer_gb300 import conforming_grad, lower_star_grad
    f = FIELDS[name]()
    base, lab, restrict, want = oracle_side(oracle, f)
    t = torch.from_numpy(f).to(gpu)
    g = lower_star_grad(t)
    assert np.array_equal(g.cpu().numpy(), base)
    asc = torch.from_numpy(lab["asc"]).to(gpu)
    dsc = torch.from_numpy(lab["dsc"]).to(gpu)
    touched, rl = conforming_grad(t, g, asc, dsc, restriction=True)
    assert np.array_equal(rl.cpu().numpy(), restrict)
    got = g.cpu().numpy()
    assert touched > 0
    assert np.array_equal(got, want), oracle_lib.describe_mismatch(got, want, f.shape[::-1])


@pytest.mark.parametrize("which", ["asc", "dsc"])
def test_conforming_grad_one_manifold(gpu, oracle, which):
    """needASC2 or needDSC2 alone: only that direction's restriction labels."""
    import torch
    from msceer_gb300 import conforming_grad, lower_star_grad
    f = FIELDS["gauss40"]()
    gt = 1e-6 * float(np.abs(f).max())
    base = oracle.grad(f)
    lab = oracle.labels(f, base, 1e-4, gt, 4000, 0.25, 0.0)
    restrict = oracle.boundary_labels(f, lab["asc"] if which == "asc" else None, lab["dsc"] if which == "dsc" else None)
    want = oracle.conform(f, restrict, base)
    t = torch.from_numpy(f).to(gpu)
    g = lower_star_grad(t)
    l = torch.from_numpy(lab[which]).to(gpu)
    conforming_grad(t, g, l if which == "asc" else None, l if which == "dsc" else None)
    assert np.array_equal(g.cpu().numpy(), want)


@pytest.mark.parametrize("name", list(FIELDS))
def test_conforming_grad_end_to_end(gpu, oracle, name):
    """The GPU labels, then the conforming .grad: differences only around the label
    differences (at most a few cells per differing vertex)."""
    import torch
    from msceer_gb300 import conforming_grad, integrated_labels, lower_star_grad
    f = FIELDS[name]()
    base, lab, restrict, want = oracle_side(oracle, f)
    t = torch.from_numpy(f).to(gpu)
    g = lower_star_grad(t)
    gt = 1e-6 * float(np.abs(f).max())
    got_lab = integrated_labels(t, g, 1e-4, gt, 4000, 0.25, 0.0)
    conforming_grad(t, g, got_lab["asc"], got_lab["dsc"])
    got = g.cpu().numpy()
    lab_diff = int((got_lab["asc"].cpu().numpy() != lab["asc"]).sum() + (got_lab["dsc"].cpu().numpy() != lab["dsc"]).sum())
    cell_diff = int((got != want).sum())
    print(name, "label differences", lab_diff, "cell differences", cell_diff)
    assert cell_diff <= 64 * lab_diff
