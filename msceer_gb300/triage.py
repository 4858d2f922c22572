"""Learned triage for the integrated labels (include/msc_triage.h).

The labeling's first pass (FP32 streamlines with path compression) is cheap; the
boundary fix-up that re-decides every vertex next to a label boundary takes about
nine tenths of the time and changes about one first-pass label in ten.  A three-layer
3x3x3 network (10 -> 16 -> 16 -> 2 channels, BF16 on the tensor cores) predicts which
first-pass labels the fix-up would change; only those vertices (plus a random audit
sample) are re-decided.  Everything here drives the library's own CUDA kernels through
the C ABI: feature extraction, forward and backward passes, the Adam step and the
triaged labeling.  The plain full integration (:func:`msceer_gb300.integrated_labels`)
is the drop-in and the yardstick of the triage's mismatch.
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from . import _lib

PARAMS = 3 * 27 * 16 * 16 + 3 * 16
NW = 27 * 16 * 16
CIN, COUT = 10, 2
WEIGHTS_FILE = Path(__file__).resolve().parent / "data" / "triage_cnn.npz"


class TriageParams(ctypes.Structure):
    """msc_triage_params (include/msc_triage.h)."""
    _fields_ = [("weights", ctypes.c_void_p), ("logit_threshold_asc", ctypes.c_float),
                ("logit_threshold_dsc", ctypes.c_float), ("audit_fraction", ctypes.c_float),
                ("audit_seed", ctypes.c_uint64)]


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _stream(dev):
    import torch
    return ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)


def _check(rc, fn):
    if rc != 0:
        lib = _lib.load()
        msg = (lib.msc_triage_last_error_string() if "forward" in fn or "backward" in fn or "adam" in fn
               else lib.msc_labels_last_error_string())
        raise _lib.MscError(rc, fn, msg.decode(errors="replace"))


def _dims(shape):
    return _lib.dims_arg(tuple(int(s) for s in shape[::-1]))


def _params(error_threshold, gradient_threshold, iteration_limit, max_step, presimp, precision):
    return _lib.IntegParams(error_threshold, gradient_threshold, iteration_limit, max_step, presimp, precision)


def init_weights(seed: int = 0):
    """He-initialised FP32 master weights on the current CUDA device (padding zero)."""
    import torch
    rng = np.random.default_rng(seed)
    p = np.zeros(PARAMS, dtype=np.float32)
    fan = [27 * CIN, 27 * 16, 27 * 16]
    for layer in range(3):
        w = rng.normal(scale=math.sqrt(2.0 / fan[layer]), size=(27, 16, 16)).astype(np.float32)
        if layer == 0:
            w[:, CIN:, :] = 0
        if layer == 2:
            w[:, :, COUT:] = 0
        p[layer * NW:(layer + 1) * NW] = w.ravel()
    return torch.from_numpy(p).cuda()


def features(f, grad, targets=True, error_threshold=1e-4, gradient_threshold=None, iteration_limit=4000,
             max_step=0.25, presimp_threshold=0.0):
    """Per direction (ascending, descending): the network features after the first pass
    (int16 [2, 16 N], row-planar BF16) and, with `targets`, where the full fix-up changes
    the first-pass label (uint8 [2, 2, N])."""
    import torch
    f = f.contiguous()
    if gradient_threshold is None:
        gradient_threshold = 1e-6 * float(f.abs().max())
    n = f.numel()
    feat = torch.empty(2, 16 * n, dtype=torch.int16, device=f.device)
    tgt = torch.empty(2, 2, n, dtype=torch.uint8, device=f.device) if targets else None
    p = _params(error_threshold, gradient_threshold, iteration_limit, max_step, presimp_threshold, 0)
    with torch.cuda.device(f.device):
        rc = _lib.load().msc_triage_features_3d(_ptr(f), _ptr(grad), _dims(f.shape), ctypes.byref(p), _ptr(feat),
                                                _ptr(tgt), _stream(f.device))
    _check(rc, "msc_triage_features_3d")
    return feat, tgt


def forward(feat, shape, weights, act1=None, act2=None):
    """Forward pass: (act1, act2, logits [2, N])."""
    import torch
    n = int(np.prod(shape))
    dev = feat.device
    if act1 is None:
        act1 = torch.empty(16 * n, dtype=torch.int16, device=dev)
    if act2 is None:
        act2 = torch.empty(16 * n, dtype=torch.int16, device=dev)
    logits = torch.empty(2 * n, dtype=torch.float32, device=dev)
    with torch.cuda.device(dev):
        rc = _lib.load().msc_triage_forward_3d(_ptr(feat), _dims(shape), _ptr(weights), _ptr(act1), _ptr(act2),
                                               _ptr(logits), _stream(dev))
    _check(rc, "msc_triage_forward_3d")
    return act1, act2, logits.view(2, n)


def backward(feat, act1, act2, logits, targets, shape, weights, pos_weight):
    """Loss and parameter gradients (FP32 [PARAMS])."""
    import torch
    dev = feat.device
    grads = torch.empty(PARAMS, dtype=torch.float32, device=dev)
    loss = torch.empty(1, dtype=torch.float64, device=dev)
    with torch.cuda.device(dev):
        rc = _lib.load().msc_triage_backward_3d(_ptr(feat), _ptr(act1), _ptr(act2), _ptr(logits.contiguous()),
                                                _ptr(targets.contiguous()), _dims(shape), _ptr(weights),
                                                ctypes.c_float(pos_weight), _ptr(grads), _ptr(loss), _stream(dev))
    _check(rc, "msc_triage_backward_3d")
    return float(loss.item()), grads


def adam_step(weights, grads, m, v, step, lr):
    import torch
    dev = weights.device
    with torch.cuda.device(dev):
        rc = _lib.load().msc_triage_adam_step(_ptr(weights), _ptr(grads), _ptr(m), _ptr(v), int(step),
                                              ctypes.c_float(lr), _stream(dev))
    _check(rc, "msc_triage_adam_step")


@dataclass
class TriageNet:
    """Trained weights (device FP32) and the decision thresholds (logits)."""
    weights: object
    threshold_asc: float = 0.0
    threshold_dsc: float = 0.0
    meta: dict = field(default_factory=dict)

    def save(self, path=WEIGHTS_FILE):
        path = Path(path)
        path.parent.mkdir(parents=True, exist_ok=True)
        np.savez(path, weights=self.weights.cpu().numpy(), threshold_asc=self.threshold_asc,
                 threshold_dsc=self.threshold_dsc, meta=np.array(repr(self.meta)))

    @classmethod
    def load(cls, path=WEIGHTS_FILE, device="cuda"):
        import torch
        z = np.load(path, allow_pickle=False)
        w = torch.from_numpy(z["weights"].astype(np.float32)).to(device)
        return cls(w, float(z["threshold_asc"]), float(z["threshold_dsc"]), {"source": str(path)})


def train(samples, steps, lr=3e-3, pos_weight=None, seed=0, weights=None, log=None):
    """Adam on a list of (feat, targets, shape) samples held on the device; one sample per
    step, cycling.  Returns the weights and the loss history."""
    import torch
    if weights is None:
        weights = init_weights(seed)
    if pos_weight is None:
        pos = sum(float(t.float().mean()) for _, t, _ in samples) / len(samples)
        pos_weight = float(min(20.0, max(1.0, (1 - pos) / max(pos, 1e-6))))
    m = torch.zeros_like(weights)
    v = torch.zeros_like(weights)
    hist = []
    for step in range(1, steps + 1):
        feat, tgt, shape = samples[(step - 1) % len(samples)]
        a1, a2, logits = forward(feat, shape, weights)
        loss, g = backward(feat, a1, a2, logits, tgt, shape, weights, pos_weight)
        adam_step(weights, g, m, v, step, lr)
        hist.append(loss)
        if log and (step % 50 == 0 or step == 1):
            log(f"step {step} loss {loss:.5f}")
    return weights, hist, pos_weight


def choose_thresholds(samples_by_dir, weights, miss_budget):
    """Per direction, the largest logit threshold (channel 0) whose unflagged positives
    stay within `miss_budget` (a fraction of all vertices) on the given samples."""
    import torch
    out = []
    for samples in samples_by_dir:
        z_pos, total = [], 0
        for feat, tgt, shape in samples:
            _, _, logits = forward(feat, shape, weights)
            z_pos.append(logits[0][tgt[0] > 0].float())
            total += logits.shape[1]
        zp = torch.sort(torch.cat(z_pos)).values
        allowed = int(miss_budget * total)
        if zp.numel() == 0:
            out.append(float("inf"))
        elif allowed >= zp.numel():
            out.append(float(zp[-1].item()) + 1.0)
        else:
            # flag logits > thr; positives with logit <= thr are missed
            out.append(float(zp[allowed].item()) - 1e-6 if allowed > 0 else float(zp[0].item()) - 1e-6)
    return out


def flagged_fraction(samples, weights, threshold):
    n, tot = 0, 0
    for feat, _, shape in samples:
        _, _, logits = forward(feat, shape, weights)
        n += int((logits[0] > threshold).sum().item())
        tot += logits.shape[1]
    return n / max(tot, 1)


def triage_labels(f, grad, net: TriageNet, error_threshold=1e-4, gradient_threshold=None, iteration_limit=4000,
                  max_step=0.25, presimp_threshold=0.0, audit_fraction=0.01, audit_seed=12345, precision=0):
    """Integrated labels with triage.  Returns {"asc", "dsc", "stats"}."""
    import torch
    f = f.contiguous()
    if gradient_threshold is None:
        gradient_threshold = 1e-6 * float(f.abs().max())
    n = f.numel()
    asc = torch.empty(n, dtype=torch.int32, device=f.device)
    dsc = torch.empty(n, dtype=torch.int32, device=f.device)
    p = _params(error_threshold, gradient_threshold, iteration_limit, max_step, presimp_threshold, precision)
    tp = TriageParams(net.weights.data_ptr(), net.threshold_asc, net.threshold_dsc, audit_fraction, audit_seed)
    stats = (ctypes.c_int64 * 8)()
    with torch.cuda.device(f.device):
        rc = _lib.load().msc_triage_labels_3d(_ptr(f), _ptr(grad), _dims(f.shape), ctypes.byref(p), ctypes.byref(tp),
                                              _ptr(asc), _ptr(dsc), stats, _stream(f.device))
    _check(rc, "msc_triage_labels_3d")
    names = ("flagged", "audited", "audit_changed", "redecided")
    st = {f"{d}_{k}": int(stats[4 * i + j]) for i, d in enumerate(("asc", "dsc")) for j, k in enumerate(names)}
    it = (ctypes.c_int64 * 6)()
    _lib.load().msc_labels_last_iterations(it)
    st.update({f"{d}_iterations_{k}": int(it[3 * i + j]) for i, d in enumerate(("asc", "dsc"))
               for j, k in enumerate(("first_pass", "fp32", "fp64"))})
    return {"asc": asc, "dsc": dsc, "stats": st}
