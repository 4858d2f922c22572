"""Seeded synthetic scalar volumes with the shapes and value distributions the
MSCEER workloads are quoted on (there is no public dataset for this path).

All volumes are float32, x fastest (numpy shape ``(Z, Y, X)`` in C order), the
layout ``RegularGridTrilinearFunction::LoadImageFromFile`` reads
(gi_regular_grid_trilinear_function.h:246-260, gi_regular_grid.h:54-56).

* :func:`gaussian_sum` -- sum of random isotropic Gaussians plus uniform noise
  (64^3 / 16 Gaussians for the bit-exact steepest_lstar check, 256^3 / 64
  Gaussians for the labeling workload).
* :func:`power_law_field` -- Gaussian random field with power spectrum
  P(k) ~ k^-3 (amplitude ~ k^-1.5), synthesised by FFT from seeded white noise,
  DC removed, normalised to zero mean / unit variance (512^3 and 8192^2 scale
  workloads, the uneven batch and the triage training set).
"""
from __future__ import annotations

import os

import numpy as np


def gaussian_sum(shape, n_gauss: int, seed: int = 0, sigma_range=(3.0, 10.0),
                 noise: float = 1e-3) -> np.ndarray:
    """``f = sum_i a_i exp(-|x - c_i|^2 / (2 sigma_i^2)) + U[-noise, noise]``.

    ``shape`` is (X, Y, Z) (or (X, Y) for 2D).  Draw order from
    ``numpy.random.default_rng(seed)``: for each Gaussian ``a ~ U[-1, 1]``, then
    the centre ``c ~ U[0, extent)`` per axis (x first), then ``sigma ~ U[lo, hi]``;
    after all Gaussians, the per-vertex noise in memory order.  Evaluated in
    float64 and rounded once to float32.
    """
    shape = tuple(int(s) for s in shape)
    rng = np.random.default_rng(seed)
    params = []
    for _ in range(n_gauss):
        a = rng.uniform(-1.0, 1.0)
        c = rng.uniform(0.0, 1.0, size=len(shape)) * np.asarray(shape, dtype=np.float64)
        s = rng.uniform(sigma_range[0], sigma_range[1])
        params.append((a, c, s))
    npshape = shape[::-1]
    axes = [np.arange(n, dtype=np.float64) for n in shape]  # x, y, (z)
    out = np.zeros(npshape, dtype=np.float64)
    for a, c, s in params:
        # separable evaluation: exp(-(dx^2+dy^2+dz^2)/2s^2) = prod of 1D factors
        fac = [np.exp(-((ax - ci) ** 2) / (2.0 * s * s)) for ax, ci in zip(axes, c)]
        if len(shape) == 3:
            out += a * (fac[2][:, None, None] * fac[1][None, :, None] * fac[0][None, None, :])
        else:
            out += a * (fac[1][:, None] * fac[0][None, :])
    if noise:
        out += rng.uniform(-noise, noise, size=npshape)
    return out.astype(np.float32)


def power_law_field(shape, seed: int = 0, exponent: float = -3.0,
                    workers: int | None = None) -> np.ndarray:
    """Gaussian random field with power spectrum ``P(k) ~ |k|^exponent``.

    White noise ``standard_normal`` from ``default_rng(seed)`` in memory order,
    real FFT, amplitude scaled by ``|k|^(exponent/2)`` (k in cycles per sample),
    the DC term zeroed, inverse FFT, then normalised to mean 0 / std 1 in float64
    and rounded to float32.  ``shape`` is (X, Y, Z) or (X, Y).
    """
    import scipy.fft as sfft

    shape = tuple(int(s) for s in shape)
    npshape = shape[::-1]
    workers = workers or os.cpu_count() or 1
    rng = np.random.default_rng(seed)
    noise = rng.standard_normal(size=npshape, dtype=np.float32)
    spec = sfft.rfftn(noise, workers=workers)
    del noise
    ks = [np.fft.fftfreq(n).astype(np.float32) for n in npshape[:-1]]
    ks.append(np.fft.rfftfreq(npshape[-1]).astype(np.float32))
    k2 = np.zeros(spec.shape, dtype=np.float32)
    for ax, k in enumerate(ks):
        sh = [1] * len(npshape)
        sh[ax] = k.size
        k2 += (k * k).reshape(sh)
    k2.flat[0] = 1.0
    amp = k2 ** np.float32(exponent / 4.0)  # |k|^(exponent/2) = (k^2)^(exponent/4)
    amp.flat[0] = 0.0
    del k2
    spec *= amp
    del amp
    field = sfft.irfftn(spec, s=npshape, workers=workers)
    del spec
    field = field.astype(np.float64)
    field -= field.mean()
    field /= field.std()
    return field.astype(np.float32)


def uneven_batch_shapes(n: int = 64, lo: int = 32, hi: int = 256, seed: int = 0):
    """Edge lengths drawn log-uniform in [lo, hi] per axis for ``n`` volumes."""
    rng = np.random.default_rng(seed)
    e = np.exp(rng.uniform(np.log(lo), np.log(hi), size=(n, 3)))
    return [tuple(int(round(v)) for v in row) for row in e]


def quantized(f: np.ndarray, levels: int) -> np.ndarray:
    """Round a field onto ``levels`` distinct values: a tie-heavy input that
    exercises the (value, then vertex index) order everywhere."""
    lo, hi = float(f.min()), float(f.max())
    q = np.floor((f - lo) / max(hi - lo, 1e-30) * (levels - 1) + 0.5)
    return q.astype(np.float32)
