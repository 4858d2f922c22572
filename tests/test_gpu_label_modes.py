"""The labels do not depend on how the work is scheduled: the fix-up ends computed
beside the first pass or per wave (MSC_EARLY_ENDS), the certain terminal regions grown
by the global frontier walk or by tile passes (MSC_TERMINAL_TILES), the descending
job's stream priority (MSC_DSC_PRIORITY) -- every combination gives the same labels bit
for bit, in both ambiguity modes of the FP32 ends (precision 0 and 2).  The switches
are read once per process, so each mode runs in a child process."""
import json
import os
import subprocess
import sys
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent

CHILD = r"""
import hashlib, json, sys
sys.path.insert(0, sys.argv[1])
import torch
from msceer_gb300 import fields, integrated_labels, lower_star_grad
shape, prec = json.loads(sys.argv[2]), int(sys.argv[3])
if len(shape) == 3 and shape[0] == 96:
    f = torch.from_numpy(fields.gaussian_sum(tuple(shape), 24, seed=3)).cuda()
else:
    f = torch.from_numpy(fields.power_law_field(tuple(shape), seed=21)).cuda()
g = lower_star_grad(f)
gt = 1e-6 * float(f.abs().max())
r = integrated_labels(f, g, error_threshold=1e-4, gradient_threshold=gt, iteration_limit=4000, max_step=0.25,
                      precision=prec)
print(json.dumps({k: hashlib.sha256(r[k].cpu().numpy().tobytes()).hexdigest() for k in ("asc", "dsc")}))
"""


def _run(env_extra, shape=(56, 48, 40), precision=0):
    env = dict(os.environ, **env_extra)
    out = subprocess.run([sys.executable, "-c", CHILD, str(ROOT), json.dumps(list(shape)), str(precision)], env=env,
                         capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    return json.loads(out.stdout.strip().splitlines()[-1])


def test_label_scheduling_modes_agree(gpu):
    base = _run({})
    for extra in ({"MSC_EARLY_ENDS": "0"}, {"MSC_TERMINAL_TILES": "1"}, {"MSC_DSC_PRIORITY": "0"},
                  {"MSC_EARLY_ENDS_CTAS": "16"}):
        assert _run(extra) == base, extra


@pytest.mark.parametrize("precision", [0, 2])
def test_early_ends_agree_gaussian_sum(gpu, precision):
    """The ends computed beside the first pass against per-wave integration on a
    Gaussian-sum volume, in both ambiguity modes, and the same labels on a second call."""
    shape = (96, 80, 72)
    base = _run({}, shape, precision)
    assert _run({}, shape, precision) == base
    assert _run({"MSC_EARLY_ENDS": "0"}, shape, precision) == base
