"""The triage network's CPU oracle checks itself: its backward pass against central
finite differences of its loss (FP64, no BF16 rounding), and its row-planar codec."""
import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parent.parent / "oracle"))
import triage_oracle as T  # noqa: E402


def small_problem(seed=0, shape=(5, 6, 7)):
    rng = np.random.default_rng(seed)
    feat = np.zeros(shape + (16,), dtype=np.float64)
    feat[..., :10] = rng.normal(size=shape + (10,))
    p = rng.normal(scale=0.2, size=T.NPARAMS)
    W, b = T.unpack(p.astype(np.float32))
    p[: T.NW].reshape(27, 16, 16)[:, 10:, :] = 0           # layer 1: 10 real inputs
    p[2 * T.NW: 3 * T.NW].reshape(27, 16, 16)[:, :, 2:] = 0  # layer 3: 2 real outputs
    p[3 * T.NW + 34:] = 0
    y = (rng.random((2,) + shape) < 0.2).astype(np.uint8)
    return feat, p, y


def test_backward_matches_finite_differences():
    feat, p, y = small_problem()
    loss, g = T.loss_and_grads(feat, p, y, 3.0, rounding=False)
    rng = np.random.default_rng(1)
    idx = np.concatenate([rng.choice(np.flatnonzero(p[:3 * T.NW] != 0), 40, replace=False),
                          3 * T.NW + np.array([0, 5, 16, 20, 32, 33])])
    eps = 1e-6
    rel = []
    for i in idx:
        q = p.copy(); q[i] += eps
        lp, _ = T.loss_and_grads(feat, q, y, 3.0, rounding=False)
        q[i] -= 2 * eps
        lm, _ = T.loss_and_grads(feat, q, y, 3.0, rounding=False)
        fd = (lp - lm) / (2 * eps)
        rel.append(abs(fd - g[i]) / (1e-4 + abs(fd)))
    # a step across a ReLU kink may spoil a few differences; the rest agree closely
    rel = np.sort(rel)
    assert rel[int(0.9 * len(rel))] < 1e-4, rel
    assert rel[-1] < 5e-2, rel


def test_bf16_rounding_ties_to_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -2.5, 3.14159], dtype=np.float32)
    r = T.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 4 * 2 ** -8 and r[3] == -2.5
    assert abs(r[4] - 3.140625) < 1e-7


def test_row_planar_roundtrip():
    rng = np.random.default_rng(2)
    a = T.bf16(rng.normal(size=(3, 4, 5, 16)).astype(np.float32))
    raw = T.to_row_planar(a)
    assert raw.size == 3 * 4 * 5 * 16
    assert np.array_equal(T.from_row_planar(raw, (5, 4, 3)), a)
