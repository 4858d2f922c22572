"""Measures the MSCEER reference's own label variation: its labeling at N OpenMP threads
against its labeling at one thread (where it is deterministic), on the fields the label
tests use and on the 256^3 64-Gaussian labeling workload.

The reference parallelises the first integration pass and the fix-up with OpenMP and
its threads race, so its multi-threaded labels differ from run to run; the fraction of
vertices that differ is the yardstick for the tolerances of the GPU label tests.  Run
on a machine with the reference sources:

    make -C oracle ref && python tests/golden/ref_label_noise.py [threads]

writes tests/golden/ref_label_noise.json (per field: the largest fraction over three
N-thread runs, integrated and final labels, ascending and descending)."""
from __future__ import annotations

import ctypes
import json
import os
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
from msceer_gb300 import fields  # noqa: E402

FIELDS = {
    "gauss40": lambda: fields.gaussian_sum((40, 36, 32), 8, seed=5),
    "k3_32": lambda: fields.power_law_field((32, 30, 28), seed=6),
    "gauss64_cfg0": lambda: fields.gaussian_sum((64, 64, 64), 16, seed=0),
    "gauss256_cfg2": lambda: fields.gaussian_sum((256, 256, 256), 64, seed=0),
}


def run(lib, f, nthreads):
    n = f.size
    asc = np.empty(n, np.int32)
    dsc = np.empty(n, np.int32)
    st = np.empty(4 * n, np.int32)
    gt = 1e-6 * float(np.abs(f).max())
    rc = lib.ref_labels_3d_threads(f.ctypes.data, *f.shape[::-1], 1e-4, gt, 4000, 0.0, asc.ctypes.data,
                                   dsc.ctypes.data, st.ctypes.data, nthreads)
    assert rc == 0
    return {"asc": asc, "dsc": dsc, "asc_integrated": st[n:2 * n].copy(), "dsc_integrated": st[3 * n:].copy()}


def main():
    nthreads = int(sys.argv[1]) if len(sys.argv) > 1 else (os.cpu_count() or 8)
    lib = ctypes.CDLL(str(ROOT / "oracle" / "_ref" / "libmsc_ref.so"))
    lib.ref_labels_3d_threads.argtypes = [ctypes.c_void_p, ctypes.c_longlong, ctypes.c_longlong, ctypes.c_longlong,
                                          ctypes.c_float, ctypes.c_float, ctypes.c_int, ctypes.c_float,
                                          ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
    out = {"threads": nthreads, "runs": 3, "fields": {}}
    for name, make in FIELDS.items():
        f = np.ascontiguousarray(make(), dtype=np.float32)
        t0 = time.time()
        one = run(lib, f, 1)
        t1 = time.time()
        worst = {k: 0.0 for k in one}
        for _ in range(3):
            many = run(lib, f, nthreads)
            for k in one:
                worst[k] = max(worst[k], float((many[k] != one[k]).mean()))
        out["fields"][name] = {"one_thread_s": round(t1 - t0, 2), **{k: v for k, v in sorted(worst.items())}}
        print(name, out["fields"][name], flush=True)
    (HERE / "ref_label_noise.json").write_text(json.dumps(out, indent=1) + "\n")


if __name__ == "__main__":
    main()
