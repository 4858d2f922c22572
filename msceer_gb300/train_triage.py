"""Train the triage network on labels the method itself generates.

    python -m msceer_gb300.train_triage [--fields 200] [--size 128] [--eval-size 512]

Training data: k^-3 Gaussian random fields (seeds 1000.., `--size`^3 vertices); for
each field and direction the library runs the first pass, records the network
features, then runs the full boundary fix-up and records where it changed the
first-pass label (the target).  The last tenth of the fields is held out to pick the
decision thresholds (per direction, the largest logit threshold that leaves at most
`--miss` of all vertices wrongly unflagged).  The trained weights and thresholds go to
msceer_gb300/data/triage_cnn.npz; an evaluation on a held-out field (seed 0,
`--eval-size`^3) reports the time of the plain and the triaged labeling and their
mismatch.  Everything runs on the library's CUDA kernels.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np


def make_samples(n, seed, integ):
    """(ascending sample, descending sample) of one field: (features, targets, shape)."""
    import torch
    from . import fields, lower_star_grad, triage
    f = torch.from_numpy(fields.power_law_field((n, n, n), seed=seed)).cuda()
    g = lower_star_grad(f)
    feat, tgt = triage.features(f, g, **integ)
    return [(feat[k].contiguous(), tgt[k].contiguous(), (n, n, n)) for k in range(2)]


def main(argv=None):
    import torch
    from . import fields, integrated_labels, lower_star_grad, triage
    ap = argparse.ArgumentParser()
    ap.add_argument("--fields", type=int, default=200)
    ap.add_argument("--size", type=int, default=128)
    ap.add_argument("--epochs", type=float, default=3.0)
    ap.add_argument("--lr", type=float, default=3e-3)
    ap.add_argument("--miss", type=float, default=4e-4, help="budget of wrongly unflagged vertices (fraction)")
    ap.add_argument("--eval-size", type=int, default=512)
    ap.add_argument("--out", default=str(triage.WEIGHTS_FILE))
    ap.add_argument("--report", default=None, help="write a JSON report here")
    a = ap.parse_args(argv)
    integ = dict(error_threshold=1e-4, gradient_threshold=None, iteration_limit=4000, max_step=0.25,
                 presimp_threshold=0.0)
    log = lambda m: print(m, flush=True)  # noqa: E731

    t0 = time.perf_counter()
    per_field = [make_samples(a.size, 1000 + i, integ) for i in range(a.fields)]
    n_val = max(1, a.fields // 10)
    train_set = [s for fs in per_field[:-n_val] for s in fs]
    val_by_dir = [[fs[k] for fs in per_field[-n_val:]] for k in range(2)]
    pos = [float(t[0].float().mean()) for fs in per_field for _, t, _ in fs]
    log(f"generated {a.fields} fields of {a.size}^3 in {time.perf_counter() - t0:.1f} s; "
        f"fraction the fix-up changes {np.mean(pos):.4f}")

    t1 = time.perf_counter()
    steps = max(1, int(a.epochs * len(train_set)))
    w, hist, pw = triage.train(train_set, steps, lr=a.lr, log=log)
    torch.cuda.synchronize()
    log(f"trained {steps} steps in {time.perf_counter() - t1:.1f} s; loss {hist[0]:.4f} -> {hist[-1]:.4f}")

    thr = triage.choose_thresholds(val_by_dir, w, a.miss)
    flagged = [triage.flagged_fraction(val_by_dir[k], w, thr[k]) for k in range(2)]
    log(f"thresholds {thr}, validation flagged fraction {flagged}")
    net = triage.TriageNet(w, thr[0], thr[1], {"fields": a.fields, "size": a.size, "steps": steps})
    net.save(a.out)

    # held-out evaluation
    n = a.eval_size
    f = torch.from_numpy(fields.power_law_field((n, n, n), seed=0)).cuda()
    g = lower_star_grad(f)
    integrated_labels(f, g, **integ)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    plain = integrated_labels(f, g, **integ)
    torch.cuda.synchronize()
    t_plain = time.perf_counter() - t2
    triage.triage_labels(f, g, net)
    torch.cuda.synchronize()
    t3 = time.perf_counter()
    tri = triage.triage_labels(f, g, net)
    torch.cuda.synchronize()
    t_tri = time.perf_counter() - t3
    mm = {k: float((tri[k] != plain[k]).float().mean()) for k in ("asc", "dsc")}
    rep = {"eval": f"{n}^3 k^-3 seed 0", "plain_s": t_plain, "triage_s": t_tri, "speedup": t_plain / t_tri,
           "mismatch_vs_plain": mm, "stats": tri["stats"], "thresholds": thr, "val_flagged": flagged,
           "loss": [hist[0], hist[-1]], "pos_weight": pw, "train_fields": len(train_set), "steps": steps}
    log(json.dumps(rep))
    if a.report:
        with open(a.report, "w") as fh:
            json.dump(rep, fh, indent=1)


if __name__ == "__main__":
    main()
