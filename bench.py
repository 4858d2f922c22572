#!/usr/bin/env python
"""Throughput of the lower-star .grad path on GB300 (one JSON line on rank 0).

Workload (default): the 512^3 float32 Gaussian random field with a k^-3 power
spectrum, seed 0 -- the scale configuration the MSCEER steepest_lstar path is
quoted on.  One step = the complete .grad of the volume (lower-star pairing +
ascending-manifold dimensions + boundary flag), bit-identical to the reference.

  value   Gvert/s with the volume already resident in HBM (CUDA events on the
          launching stream, K steps between barriers + synchronisation, max over
          ranks; every rank runs its own replica -- the path needs no collective)
  e2e     the same metric through the C ABI host entry (msc_steepest_lstar_host)
          with pinned host buffers: H2D of f, compute, D2H of the .grad per step
  roofline  the dominant kernel's algorithmic bytes / its measured duration
          against the measured HBM copy bandwidth (MEASURED_PEAKS.json)
  cpu_baseline  the CPU port of the reference algorithm (oracle/) on a bounded
          z-slab sample of the same volume, all host threads

`--impl reference` times the reference's CPU algorithm alone (the port: the
reference's own sources are not on the GPU host) on the same metric.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

METRIC = "Gvert/s: lower-star .grad + integrated labels, learned vs plain @<=0.1% mismatch"
UNIT = "Gvert/s"
L2_BYTES = 129 * 1024 * 1024


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--size", type=int, default=512, help="edge of the cubic volume")
    p.add_argument("--no-cpu-baseline", action="store_true")
    return p.parse_args()


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def load_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def make_volume(n: int, seed: int = 0) -> np.ndarray:
    from msceer_gb300 import fields
    cache = Path(tempfile.gettempdir()) / f"msc_k3_{n}_{seed}.f32"
    if cache.exists() and cache.stat().st_size == 4 * n ** 3:
        return np.fromfile(cache, dtype=np.float32).reshape(n, n, n)
    f = fields.power_law_field((n, n, n), seed=seed)
    try:
        f.tofile(cache)
    except OSError:
        pass
    return f


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_id: str | None):
        self.gpu_id = gpu_id
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            cmd = ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "100"]
            if self.gpu_id:
                cmd += ["--id", self.gpu_id]
            self.proc = subprocess.Popen(cmd, stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.proc is None or not self.path:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        rows = []
        for line in Path(self.path).read_text().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def cpu_baseline(f: np.ndarray, slab: int, reps: int = 1):
    """The oracle port of the reference algorithm on a z-slab of the volume."""
    import oracle_lib
    orc = oracle_lib.load()
    sample = np.ascontiguousarray(f[:slab])
    nthreads = os.cpu_count() or 1
    times = []
    for _ in range(reps):
        t0 = time.perf_counter()
        orc.grad(sample, nthreads=nthreads)
        times.append(time.perf_counter() - t0)
    t = statistics.median(times)
    nv = sample.size
    return {"value": nv / t / 1e9, "unit": UNIT, "cores": nthreads, "kind": "port",
            "sample": f"z-slab {sample.shape[2]}x{sample.shape[1]}x{sample.shape[0]} of the volume "
                      f"({nv} vertices), oracle/msc_oracle.c with {nthreads} OpenMP threads, "
                      f"median of {reps}: {t:.2f} s"}


def run_reference(args, ws, rank):
    if rank != 0:
        return
    f = make_volume(args.size)
    slab = max(2, args.size // 8)
    vals = []
    for i in range(args.warmup + args.steps):
        r = cpu_baseline(f, slab)
        if i >= args.warmup:
            vals.append(r["value"])
    v = statistics.mean(vals)
    nv = f[:slab].size
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": nv / (v * 1e9) * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": f"steepest_lstar .grad, {args.size}^3 k^-3 GRF seed 0",
                       "sample": f"z-slab of {slab} planes per step"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": r["cores"], "kind": "port",
                             "sample": r["sample"]},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args, ws, rank, local):
    import torch
    from msceer_gb300 import _lib, ascending_manifold_dims, lower_star_grad, lower_star_pairs, num_cells

    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    pg = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
        pg = dist
    lib = _lib.load()

    n = args.size
    f_np = make_volume(n, seed=rank)  # each replica its own volume
    dims = (n, n, n)
    V = n ** 3
    C = num_cells(dims)
    f_host = torch.from_numpy(f_np).pin_memory()
    f_dev = f_host.to(dev)
    g_dev = torch.empty(C, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)

    def barrier():
        if pg is not None:
            pg.barrier()
        torch.cuda.synchronize(dev)

    for _ in range(args.warmup):
        lower_star_grad(f_dev, out=g_dev)
    passes = lib.msc_last_ldir_passes()
    barrier()

    gpu_id = None
    try:
        gpu_id = "GPU-" + str(torch.cuda.get_device_properties(dev).uuid)
    except Exception:
        gpu_id = None
    with ClockSampler(gpu_id) as clk:
        barrier()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        total_passes = 0
        for _ in range(args.steps):
            lower_star_grad(f_dev, out=g_dev)
            total_passes += lib.msc_last_ldir_passes()
        e1.record(stream)
        barrier()
    ms = e0.elapsed_time(e1) / args.steps
    clocks = clk.summary()
    if pg is not None:
        t = torch.tensor([ms], device=dev)
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
        ms = float(t.item())
    value = ws * V / (ms * 1e-3) / 1e9

    # per-stage breakdown on the launching stream
    reps = max(3, args.steps)
    s0, s1, s2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    t_pairs = t_ldir = 0.0
    npass = 0
    for _ in range(reps):
        s0.record(stream)
        lower_star_pairs(f_dev, out=g_dev)
        s1.record(stream)
        npass += ascending_manifold_dims(g_dev, dims)
        s2.record(stream)
        torch.cuda.synchronize(dev)
        t_pairs += s0.elapsed_time(s1)
        t_ldir += s1.elapsed_time(s2)
    t_pairs /= reps
    t_ldir_pass = t_ldir / npass
    t_ldir /= reps

    # end to end through the C ABI host entry, pinned host buffers
    g_host = torch.empty(C, dtype=torch.uint8).pin_memory()
    fptr = ctypes.c_void_p(f_host.data_ptr())
    gptr = ctypes.c_void_p(g_host.data_ptr())
    dptr = _lib.dims_arg(dims)
    _lib.check(lib.msc_steepest_lstar_host(fptr, dptr, gptr), "msc_steepest_lstar_host")
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        _lib.check(lib.msc_steepest_lstar_host(fptr, dptr, gptr), "msc_steepest_lstar_host")
    t_e2e = (time.perf_counter() - t0) / args.steps
    if pg is not None:
        t = torch.tensor([t_e2e], device=dev)
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
        t_e2e = float(t.item())
    e2e = ws * V / t_e2e / 1e9
    assert torch.equal(g_host.to(dev), g_dev), "host and device paths disagree"

    peak, peak_kind = load_peaks()
    alg_pairs = 4 * V + C            # read f once, write every .grad byte once
    alg_pass = 2 * C                 # one ascending-manifold pass reads and writes the .grad
    kernels = {
        "lstar_kernel": {"launches_per_step": 1, "ms_per_launch": t_pairs,
                         "algorithmic_bytes": alg_pairs, "gbs": alg_pairs / (t_pairs * 1e-3) / 1e9},
        "ldir_pass_kernel": {"launches_per_step": npass / reps, "ms_per_launch": t_ldir_pass,
                             "algorithmic_bytes": alg_pass, "gbs": alg_pass / (t_ldir_pass * 1e-3) / 1e9},
    }
    dom = max(kernels, key=lambda k: kernels[k]["ms_per_launch"] * kernels[k]["launches_per_step"])
    kd = kernels[dom]
    traffic = TRAFFIC_PER_LAUNCH.get((dom, n))
    roofline = {"kernel": dom, "bound": "hbm", "achieved": kd["gbs"], "peak": peak, "unit": "GB/s",
                "frac": kd["gbs"] / peak, "peak_kind": f"{peak_kind} hbm_gbs",
                "traffic": traffic}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": f"steepest_lstar .grad (lower star + ldir + flag), {n}^3 float32 "
                                       f"k^-3 Gaussian random field, seed = rank",
                           "vertices": V, "cells": C, "parallelism": f"replicas x{ws}",
                           "l2": "inputs larger than L2 (f 512 MiB, .grad 1 GiB at 512^3); no flush"},
                "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": 4 * V, "d2h_bytes_per_step": C,
                        "ms_per_step": t_e2e * 1e3, "api": "msc_steepest_lstar_host"},
                "roofline": roofline,
                "kernels": kernels,
                "gpu_launches": args.steps * 1 + total_passes,
                "clocks": clocks}
        if ws == 1 and not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline(f_np, max(2, n // 8))
        print(json.dumps(line), flush=True)
    if pg is not None:
        pg.destroy_process_group()


# dram__bytes_read.sum + dram__bytes_write.sum per launch from the committed ncu
# summaries under profiles/ (None until captured)
TRAFFIC_PER_LAUNCH: dict = {}


def main():
    args = parse_args()
    ws, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, ws, rank)
    else:
        run_ours(args, ws, rank, local)


if __name__ == "__main__":
    main()
