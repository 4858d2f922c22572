#!/usr/bin/env python
"""Throughput of the .grad + integrated-labels path on GB300 (one JSON line on rank 0).

Workload (default): the 512^3 float32 Gaussian random field with a k^-3 power
spectrum, seed = rank (held out from the triage network's training fields).  One
step = the complete lower-star .grad of the volume (bit-identical to steepest_lstar)
plus the ascending and descending integrated labels of ondemandaccurate (error
threshold 1e-4, gradient threshold 1e-6 max|f|, 4000 iterations, 0.25-voxel steps)
through the plain full integration; the learned triage (when its trained weights are
present) is measured beside it ("learned": throughput, speed-up and label difference
against the plain labels), or timed as the step with --triage.

  value       Gvert/s of the step with the volume already resident in HBM (CUDA
              events on the launching stream, K steps between barriers +
              synchronisation, max over ranks; every rank runs its own replica --
              the path needs no collective)
  plain       the step with the plain full integration (the drop-in path, and the
              yardstick of the triage)
  learned     the step with the learned triage, its speed-up over plain and its
              label difference from the plain labels
  e2e         the same metric through the C ABI host entry msc_ondemand_labels_host:
              H2D of f, .grad, labels, D2H of both label volumes per step
  grad        the .grad alone: Gvert/s and its per-kernel breakdown
  grad_2d     the .grad of the 8192^2 k^-3 field (2D): Gvert/s, kernels, roofline
  conforming_grad  ondemandaccurate's accurate 3-manifold .grad of the step (restriction
              labels from its final labels, re-pairing, ldir): ms, touched vertices
  ms_graph    the Morse-Smale complex nodes and arcs of the step's .grad on the device
              (msc_ms_graph_3d, extractmsc's arc flags): counts, ms, Gvert/s
  roofline    the dominant .grad kernel's algorithmic bytes / its measured duration
              against the measured HBM copy bandwidth (MEASURED_PEAKS.json)
  mismatch_vs_fp64_oracle  the labeling workload (256^3, 64 Gaussians, seed 0): the
              fraction of vertices whose plain / learned labels differ from the FP64
              oracle's (the reference's one-thread algorithm, run on the host during
              the timing), beside the reference's own 8-thread-vs-1-thread variation
  cpu_baseline  the CPU port of the reference algorithm (oracle/) on bounded samples
              of the same volume: .grad on a z-slab (all threads), labels of full
              x-y slabs (one single-threaded process per core)

`--impl reference` times the reference's CPU algorithm alone (the port: the
reference's own sources are not on the GPU host) on the same metric.
`--grad-only` times the .grad alone (`--2d`: of the 8192^2 field); `--workload labels`
makes the 256^3 labeling workload the step.
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
INTEG = dict(error_threshold=1e-4, iteration_limit=4000, max_step=0.25, presimp_threshold=0.0)


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--size", type=int, default=512, help="edge of the cubic volume")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--triage", action="store_true",
                   help="time the learned triage as the step (default: the plain full integration, with the triage "
                        "measured beside it)")
    p.add_argument("--no-triage", action="store_true", help="skip the learned triage altogether")
    p.add_argument("--grad-only", action="store_true", help="time the .grad alone as the step")
    p.add_argument("--no-batch", action="store_true", help="skip the 64-volume batching measurement")
    p.add_argument("--2d", dest="two_d", action="store_true", help="with --grad-only: the 8192^2 .grad")
    p.add_argument("--workload", choices=["k3", "labels"], default="k3",
                   help="k3: the 512^3 k^-3 field (default); labels: the 256^3 64-Gaussian labeling workload")
    p.add_argument("--no-oracle", action="store_true", help="skip the FP64-oracle label comparison")
    return p.parse_args()


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(x: float, pg, device) -> float:
    """The largest value of x over the ranks (the slowest replica's time)."""
    if pg is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def aggregate_gvps(ws: int, vertices_per_rank: int, seconds: float) -> float:
    """Whole-job Gvert/s: every rank processes its own volume in `seconds` (the max over ranks)."""
    return ws * vertices_per_rank / seconds / 1e9


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


NOISE_FILE = ROOT / "tests" / "golden" / "ref_label_noise.json"


def labels_field(seed: int = 0) -> np.ndarray:
    """The labeling workload: 256^3 float32, 64 Gaussians + U[-1e-3, 1e-3] noise."""
    from msceer_gb300 import fields
    return fields.gaussian_sum((256, 256, 256), 64, seed=seed)


def _oracle_labels_job(path: str, q) -> None:
    """FP64 oracle labels of the labeling workload (a spawned process): the reference's
    one-thread algorithm, written to `path`; its labeling time goes to `q`."""
    import oracle_lib
    f = labels_field()
    orc = oracle_lib.load()
    g = orc.grad(f, nthreads=0)
    gt = 1e-6 * float(np.abs(f).max())
    t0 = time.perf_counter()
    lab = orc.labels(f, g, INTEG["error_threshold"], gt, INTEG["iteration_limit"], INTEG["max_step"],
                     INTEG["presimp_threshold"])
    np.savez(path, asc=lab["asc"], dsc=lab["dsc"])
    q.put(time.perf_counter() - t0)


def _label_crop_worker(args):
    """One oracle labeling of a sub-volume (run in a spawned process)."""
    crop, = args
    import oracle_lib
    orc = oracle_lib.load()
    g = orc.grad(crop, nthreads=1)
    gt = 1e-6 * float(np.abs(crop).max())
    t0 = time.perf_counter()
    orc.labels(crop, g, INTEG["error_threshold"], gt, INTEG["iteration_limit"], INTEG["max_step"],
               INTEG["presimp_threshold"])
    return crop.size, time.perf_counter() - t0


def cpu_baseline(f: np.ndarray, grad_only: bool = False):
    """The oracle port of the reference algorithm on bounded samples of the volume:
    the .grad of a z-slab with all host threads, and the labels (single-threaded
    restatement) of one 40^3 sub-volume per host core in parallel processes."""
    import multiprocessing as mp

    import oracle_lib
    orc = oracle_lib.load()
    n = f.shape[0]
    slab = np.ascontiguousarray(f[: max(2, n // 8)])
    nthreads = os.cpu_count() or 1
    t0 = time.perf_counter()
    orc.grad(slab, nthreads=nthreads)
    t_grad = time.perf_counter() - t0
    g_grad = slab.size / t_grad / 1e9
    out = {"unit": UNIT, "cores": nthreads, "kind": "port", "grad_gvps": g_grad}
    shape = "x".join(str(e) for e in slab.shape[::-1])
    desc = (f".grad of a {'z-slab' if slab.ndim == 3 else 'y-band'} {shape} ({slab.size} vertices) with "
            f"{nthreads} OpenMP threads: {t_grad:.2f} s")
    if grad_only:
        out["value"] = g_grad
        out["sample"] = desc
        return out
    c = 4  # z-planes per slab: full x-y extent, so streamlines run as long as in the volume
    crops = []
    for i in range(nthreads):
        z0 = (i * (n - c)) // max(1, nthreads - 1) if nthreads > 1 else 0
        crops.append((np.ascontiguousarray(f[z0:z0 + c]),))
    ctx = mp.get_context("spawn")
    t1 = time.perf_counter()
    with ctx.Pool(nthreads) as pool:
        res = pool.map(_label_crop_worker, crops)
    wall = time.perf_counter() - t1
    nv = sum(r[0] for r in res)
    busy = max(r[1] for r in res)
    g_lab = nv / busy / 1e9
    out["labels_gvps"] = g_lab
    out["value"] = 1.0 / (1.0 / g_grad + 1.0 / g_lab)
    out["sample"] = (desc + f"; labels (FP64 oracle, one thread each) of {len(crops)} z-slabs "
                     f"{f.shape[2]}x{f.shape[1]}x{c} in {len(crops)} spawned processes, slowest {busy:.2f} s "
                     f"(pool wall {wall:.2f} s); value = harmonic combination of the two rates")
    return out


def bench_volume(args, rank):
    """The step's volume: (f, dims (x, y[, z]), edge, description)."""
    if args.grad_only and args.two_d:
        from msceer_gb300 import fields
        return fields.power_law_field((8192, 8192), seed=rank), (8192, 8192), 8192, \
            "8192^2 float32 k^-3 Gaussian random field"
    if args.workload == "labels":
        return labels_field(seed=rank), (256, 256, 256), 256, \
            "256^3 float32 sum of 64 Gaussians + noise (the labeling workload)"
    n = args.size
    return make_volume(n, seed=rank), (n, n, n), n, f"{n}^3 float32 k^-3 Gaussian random field"


def run_reference(args, ws, rank):
    if rank != 0:
        return
    f, dims, n, wl_name = bench_volume(args, 0)
    vals = []
    r = None
    for i in range(args.warmup + args.steps):
        r = cpu_baseline(f, grad_only=args.grad_only)
        if i >= args.warmup:
            vals.append(r["value"])
    v = statistics.mean(vals)
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32" if args.grad_only else "f32+f64",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": f"{'.grad' if args.grad_only else '.grad + integrated labels'}, "
                                   f"{wl_name}, seed 0, bounded CPU samples per step",
                       "sample": r["sample"]},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": r["cores"], "kind": "port", "sample": r["sample"]},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def _events(n):
    import torch
    return [torch.cuda.Event(enable_timing=True) for _ in range(n)]


def grad_stage_times(f_dev, g_dev, dims, reps, stream, dev):
    """CUDA-event times (ms) of the .grad's two stages and of the whole .grad, averaged
    over `reps` runs, and the ldir stage's kernel launches over those runs."""
    import torch
    from msceer_gb300 import ascending_manifold_dims, lower_star_grad, lower_star_pairs
    s0, s1, s2 = _events(3)
    t_pairs = t_ldir = t_grad = 0.0
    nlaunch = 0
    for _ in range(reps):
        s0.record(stream)
        lower_star_pairs(f_dev, out=g_dev)
        s1.record(stream)
        nlaunch += ascending_manifold_dims(g_dev, dims)
        s2.record(stream)
        torch.cuda.synchronize(dev)
        t_pairs += s0.elapsed_time(s1)
        t_ldir += s1.elapsed_time(s2)
    for _ in range(reps):
        s0.record(stream)
        lower_star_grad(f_dev, out=g_dev)
        s1.record(stream)
        torch.cuda.synchronize(dev)
        t_grad += s0.elapsed_time(s1)
    return t_pairs / reps, t_ldir / reps, t_grad / reps, nlaunch


def grad_kernels(V, C, t_pairs, t_ldir, nlaunch, reps, n, peak, peak_kind):
    """Per-stage algorithmic bandwidth of the .grad and the roofline of its dominant stage."""
    alg_pairs = 4 * V + C            # read f once, write every .grad byte once
    alg_ldir = 2 * C                 # the ascending-manifold stage reads and writes the .grad
    kernels = {
        "lstar_kernel": {"launches_per_step": 1, "ms_per_launch": t_pairs,
                         "algorithmic_bytes": alg_pairs, "gbs": alg_pairs / (t_pairs * 1e-3) / 1e9},
        "ldir_stage": {"launches_per_step": nlaunch / reps, "ms_per_stage": t_ldir,
                       "algorithmic_bytes": alg_ldir, "gbs": alg_ldir / (t_ldir * 1e-3) / 1e9,
                       "kernels": "ldir_tile_kernel + ldir_check_kernel + ldir_walk_kernel"},
    }
    dom = "lstar_kernel" if t_pairs >= t_ldir else "ldir_stage"
    kd = kernels[dom]
    roofline = {"kernel": dom, "bound": "hbm", "achieved": kd["gbs"], "peak": peak, "unit": "GB/s",
                "frac": kd["gbs"] / peak, "peak_kind": f"{peak_kind} hbm_gbs", "traffic": TRAFFIC_PER_LAUNCH.get((dom, n)),
                "scope": "dominant kernel of the .grad; the label integration that dominates the full step is "
                         "FP32/FP64 issue-bound, neither HBM nor tensor bound"}
    # the bound these kernels actually meet: instruction issue (per-unit counts from ncu)
    per, unit = WARP_INST_PER_UNIT[dom]
    units = V if unit == "vertex" else C
    t = kd.get("ms_per_launch", kd.get("ms_per_stage")) * 1e-3
    issue_peak = SMS * SCHEDULERS_PER_SM * SM_MAX_MHZ * 1e6
    roofline["issue"] = {"warp_inst_per_" + unit: per, "achieved_warp_inst_per_s": per * units / t,
                         "peak_warp_inst_per_s": issue_peak, "frac": per * units / t / issue_peak,
                         "source": "smsp__inst_executed.sum of the 256^3 ncu capture x units / CUDA-event time"}
    return kernels, roofline


def run_ours(args, ws, rank, local):
    import torch
    from msceer_gb300 import _lib, integrated_labels, lower_star_grad, num_cells, triage

    # the FP64 oracle of the labeling workload runs on the host while the GPU is timed
    oracle_job = None
    if rank == 0 and not args.grad_only and not args.no_oracle:
        import multiprocessing as mp
        ctx = mp.get_context("spawn")
        oq = ctx.Queue()
        opath = os.path.join(tempfile.mkdtemp(prefix="msc_oracle_"), "labels.npz")
        oproc = ctx.Process(target=_oracle_labels_job, args=(opath, oq))
        oproc.start()
        oracle_job = (oproc, oq, opath)

    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    pg = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
        pg = dist
    lib = _lib.load()

    f_np, dims, n, wl_name = bench_volume(args, rank)  # each replica its own volume
    V = int(np.prod(dims))
    C = num_cells(dims)
    f_host = torch.from_numpy(f_np).pin_memory()
    f_dev = f_host.to(dev)
    g_dev = torch.empty(C, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    gt = 1e-6 * float(np.abs(f_np).max())
    integ = dict(INTEG, gradient_threshold=gt)

    net = None  # the trained triage network, measured beside the step (or as the step with --triage)
    if not args.grad_only and not args.no_triage and triage.WEIGHTS_FILE.exists():
        net = triage.TriageNet.load(device=dev)
    step_net = net if args.triage else None

    def step():
        lower_star_grad(f_dev, out=g_dev)
        if args.grad_only:
            return None
        if step_net is not None:
            return triage.triage_labels(f_dev, g_dev, step_net, **integ)
        return integrated_labels(f_dev, g_dev, **integ)

    def barrier():
        if pg is not None:
            pg.barrier()
        torch.cuda.synchronize(dev)

    for _ in range(args.warmup):
        step()
    barrier()

    gpu_id = None
    try:
        gpu_id = "GPU-" + str(torch.cuda.get_device_properties(dev).uuid)
    except Exception:
        gpu_id = None
    with ClockSampler(gpu_id) as clk:
        barrier()
        e0, e1 = _events(2)
        l0 = lib.msc_kernel_launches()
        e0.record(stream)
        res = None
        for _ in range(args.steps):
            res = step()
        e1.record(stream)
        barrier()
        launches = lib.msc_kernel_launches() - l0
    ms = max_over_ranks(e0.elapsed_time(e1) / args.steps, pg, dev)
    clocks = clk.summary()
    value = aggregate_gvps(ws, V, ms * 1e-3)

    # end to end through the C ABI host entry, pinned host buffers, right after the step
    # (the same conditions: the oracle job on the host, no other measurement before it)
    e2e_reps = max(1, args.steps)
    if args.grad_only:
        g_host = torch.empty(C, dtype=torch.uint8).pin_memory()
        api = "msc_steepest_lstar_host" if len(dims) == 3 else "msc_lower_star_grad_2d_host"
        fn = lambda: _lib.check(getattr(lib, api)(ctypes.c_void_p(f_host.data_ptr()), _lib.dims_arg(dims),  # noqa: E731
                                                  ctypes.c_void_p(g_host.data_ptr())), api)
        h2d, d2h = 4 * V, C
    else:
        a_host = torch.empty(V, dtype=torch.int32).pin_memory()
        d_host = torch.empty(V, dtype=torch.int32).pin_memory()
        p = _lib.IntegParams(integ["error_threshold"], gt, integ["iteration_limit"], integ["max_step"],
                             integ["presimp_threshold"], 0)
        tp = None
        if step_net is not None:
            tp = triage.TriageParams(step_net.weights.data_ptr(), step_net.threshold_asc, step_net.threshold_dsc,
                                     0.01, 12345)

        def fn():
            rc = lib.msc_ondemand_labels_host(ctypes.c_void_p(f_host.data_ptr()), _lib.dims_arg(dims), ctypes.byref(p),
                                              ctypes.byref(tp) if tp is not None else None,
                                              ctypes.c_void_p(a_host.data_ptr()), ctypes.c_void_p(d_host.data_ptr()))
            _lib.check(rc, "msc_ondemand_labels_host")
        h2d, d2h, api = 4 * V, 8 * V, "msc_ondemand_labels_host"
    fn()
    barrier()
    e2e_ms = []
    t0 = time.perf_counter()
    for _ in range(e2e_reps):
        t1 = time.perf_counter()
        fn()
        e2e_ms.append((time.perf_counter() - t1) * 1e3)
    t_e2e = max_over_ranks((time.perf_counter() - t0) / e2e_reps, pg, dev)
    e2e = aggregate_gvps(ws, V, t_e2e)

    # the .grad alone and its stages, on the launching stream
    reps = max(3, min(args.steps, 10))
    t_pairs, t_ldir, t_grad, nlaunch = grad_stage_times(f_dev, g_dev, dims, reps, stream, dev)

    line_extra = {}
    if not args.grad_only:
        # the other mode with the same warm-up and step count (the plain full
        # integration beside a triaged step, or the triage beside the plain step) and the
        # triage's label difference from the plain labels
        def timed(use_net):
            def one():
                lower_star_grad(f_dev, out=g_dev)
                return triage.triage_labels(f_dev, g_dev, use_net, **integ) if use_net is not None else \
                    integrated_labels(f_dev, g_dev, **integ)
            for _ in range(args.warmup):
                one()
            torch.cuda.synchronize(dev)
            p0, p1 = _events(2)
            p0.record(stream)
            for _ in range(args.steps):
                r = one()
            p1.record(stream)
            torch.cuda.synchronize(dev)
            return r, p0.elapsed_time(p1) / args.steps
        if step_net is not None:
            plain, ms_plain = timed(None)
            learned, ms_learned = res, ms
        else:
            plain, ms_plain = res, ms
            learned, ms_learned = timed(net) if net is not None else (None, None)
        line_extra["plain"] = {"value": V / (ms_plain * 1e-3) / 1e9, "unit": UNIT, "ms_per_step": ms_plain,
                               "redecided": plain["stats"]}
        line_extra["labels"] = {"mode": "learned triage" if step_net is not None else "plain full integration"}
        if learned is not None:
            line_extra["learned"] = {
                "value": V / (ms_learned * 1e-3) / 1e9, "unit": UNIT, "ms_per_step": ms_learned,
                "speedup_vs_plain": ms_plain / ms_learned,
                "mismatch_vs_plain": {k: float((learned[k] != plain[k]).float().mean().item()) for k in ("asc", "dsc")},
                "stats": learned["stats"], "thresholds": [net.threshold_asc, net.threshold_dsc]}
        # the labeling's kernels are FP32 issue-bound streamline integrations: their
        # roofline is the FP32 rate.  Operations per advection iteration: two trilinear
        # interpolations of the 3-vector gradient (73 each) plus step control (~37).
        st = res["stats"]
        it32 = sum(st.get(f"{d}_iterations_{k}", 0) for d in ("asc", "dsc") for k in ("first_pass", "fp32"))
        it64 = sum(st.get(f"{d}_iterations_fp64", 0) for d in ("asc", "dsc"))
        labels_ms = max(ms - t_grad, 1e-9)
        sms = torch.cuda.get_device_properties(dev).multi_processor_count
        fp32_peak = FP32_LANES_PER_SM * sms * 2 * SM_MAX_MHZ * 1e6 / 1e12
        achieved = it32 * FLOP_PER_ITERATION / (labels_ms * 1e-3) / 1e12
        line_extra["integration"] = {
            "kernels": "speculate_kernel + fixup_end32_kernel (FP32), fixup_end64_kernel (FP64 re-decisions)",
            "bound": "fp32 issue", "iterations_fp32": it32, "iterations_fp64": it64,
            "flop_per_iteration": FLOP_PER_ITERATION, "labels_ms": labels_ms,
            "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s", "frac": achieved / fp32_peak,
            "peak_kind": f"nominal FP32 ({sms} SMs x {FP32_LANES_PER_SM} lanes x FMA at {SM_MAX_MHZ} MHz)",
            "scope": "all FP32 advection iterations of the step over the whole labeling time (every labeling "
                     "kernel included, so a lower bound for the integration kernels)"}

    # batching: 64 volumes with edge lengths log-uniform in [32, 256] per axis (k^-3 fields,
    # seeds 0..63): the .grad of all of them in shared launches vs one call per volume
    batch = None
    if not args.no_batch:
        from msceer_gb300 import fields, lower_star_grad_batch
        rng = np.random.default_rng(0)
        shapes = [tuple(int(round(np.exp(rng.uniform(np.log(32), np.log(256))))) for _ in range(3)) for _ in range(64)]
        vols = [torch.from_numpy(fields.power_law_field(sh, seed=i)).to(dev) for i, sh in enumerate(shapes)]
        nvb = sum(int(np.prod(sh)) for sh in shapes)
        outs = lower_star_grad_batch(vols)
        singles = [lower_star_grad(v) for v in vols]
        same = all(torch.equal(a, b) for a, b in zip(outs, singles))
        b0, b1, b2 = _events(3)
        b0.record(stream)
        for _ in range(3):
            lower_star_grad_batch(vols, outs)
        b1.record(stream)
        for _ in range(3):
            for v, o in zip(vols, singles):
                lower_star_grad(v, out=o)
        b2.record(stream)
        torch.cuda.synchronize(dev)
        tb, tl = b0.elapsed_time(b1) / 3, b1.elapsed_time(b2) / 3
        batch = {"workload": "64 k^-3 volumes, edges log-uniform in [32, 256], seeds 0..63, .grad",
                 "vertices": nvb, "batched": {"value": nvb / (tb * 1e-3) / 1e9, "unit": UNIT, "ms": tb},
                 "looped": {"value": nvb / (tl * 1e-3) / 1e9, "unit": UNIT, "ms": tl}, "bit_identical": same}
        # the labels of the same volumes: several volumes at a time on their own streams
        # against one call after another, and the whole .grad + labels step of the batch
        from msceer_gb300 import integrated_labels_batch
        lab_kw = dict(INTEG)
        integrated_labels_batch(vols, outs, threads=8, **lab_kw)
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        lab_b = integrated_labels_batch(vols, outs, threads=8, **lab_kw)
        torch.cuda.synchronize(dev)
        tlb = time.perf_counter() - t0
        t0 = time.perf_counter()
        lab_l = [integrated_labels(v, o, **lab_kw) for v, o in zip(vols, outs)]
        torch.cuda.synchronize(dev)
        tll = time.perf_counter() - t0
        same_l = all(torch.equal(a[k], b[k]) for a, b in zip(lab_b, lab_l) for k in ("asc", "dsc"))
        batch["labels"] = {"how": "8 volumes at a time on their own CUDA streams and host threads vs one call "
                                  "after another (each call synchronises only its own stream)",
                           "batched": {"value": nvb / tlb / 1e9, "unit": UNIT, "ms": tlb * 1e3},
                           "looped": {"value": nvb / tll / 1e9, "unit": UNIT, "ms": tll * 1e3},
                           "bit_identical": same_l,
                           "step": {"what": ".grad batched + labels batched", "value": nvb / (tb * 1e-3 + tlb) / 1e9,
                                    "unit": UNIT}}
        del vols, outs, singles, lab_b, lab_l

    peak, peak_kind = load_peaks()
    kernels, roofline = grad_kernels(V, C, t_pairs, t_ldir, nlaunch, reps, n, peak, peak_kind)

    # the 2D scale workload: the .grad of the 8192^2 k^-3 field
    grad_2d = None
    if not args.grad_only and not args.no_batch:
        from msceer_gb300 import fields
        f2 = torch.from_numpy(fields.power_law_field((8192, 8192), seed=rank)).to(dev)
        g2 = torch.empty(num_cells((8192, 8192)), dtype=torch.uint8, device=dev)
        for _ in range(args.warmup):
            lower_star_grad(f2, out=g2)
        p2, l2, t2, nl2 = grad_stage_times(f2, g2, (8192, 8192), reps, stream, dev)
        V2, C2 = 8192 * 8192, num_cells((8192, 8192))
        k2, r2 = grad_kernels(V2, C2, p2, l2, nl2, reps, 8192, peak, peak_kind)
        grad_2d = {"workload": "8192^2 float32 k^-3 Gaussian random field, seed = rank", "vertices": V2, "cells": C2,
                   "value": V2 / (t2 * 1e-3) / 1e9, "unit": UNIT, "ms_per_step": t2, "kernels": k2, "roofline": r2}
        del f2, g2

    # ondemandaccurate's accurate 3-manifold .grad of the step: restriction labels from
    # the step's final labels, the re-pairing of the touched vertices, the ldir stage
    conform = None
    if not args.grad_only and not args.no_batch and isinstance(res, dict) and "asc" in res:
        from msceer_gb300 import conforming_grad
        lower_star_grad(f_dev, out=g_dev)
        base = g_dev.clone()
        touched = conforming_grad(f_dev, g_dev, res["asc"], res["dsc"])
        torch.cuda.synchronize(dev)
        tc = 0.0
        for _ in range(reps):
            g_dev.copy_(base)
            c0, c1 = _events(2)
            c0.record(stream)
            conforming_grad(f_dev, g_dev, res["asc"], res["dsc"])
            c1.record(stream)
            torch.cuda.synchronize(dev)
            tc += c0.elapsed_time(c1)
        tc /= reps
        conform = {"workload": "msc_conforming_grad_3d on the step's .grad with its final labels (needASC2 = "
                               "needDSC2 = 1)", "touched_vertices": int(touched), "ms": tc,
                   "value": V / (tc * 1e-3) / 1e9, "unit": UNIT}
        del base

    # the Morse-Smale complex graph of the bench volume's .grad (extractmsc's
    # ComputeFromGrad: arcs from 1-saddles and maxima, no geometry)
    graph = None
    if not args.no_batch:
        from msceer_gb300 import ms_graph
        lower_star_grad(f_dev, out=g_dev)
        res = ms_graph(g_dev, f_dev, (1, 0, 1))
        torch.cuda.synchronize(dev)
        m0, m1 = _events(2)
        m0.record(stream)
        for _ in range(reps):
            res = ms_graph(g_dev, f_dev, (1, 0, 1))
        m1.record(stream)
        torch.cuda.synchronize(dev)
        tg = m0.elapsed_time(m1) / reps
        graph = {"workload": f"MorseSmaleComplexBasic::ComputeFromGrad of the step's .grad, arcs from 1-saddles "
                             f"and maxima (extractmsc's flags), no arc geometry",
                 "nodes": int(res["node_cell"].numel()), "arcs": int(res["arc_lower"].numel()), "ms": tg,
                 "value": V / (tg * 1e-3) / 1e9, "unit": UNIT}
        del res

    # the labeling workload against the FP64 oracle: plain and learned labels
    mismatch = None
    if oracle_job is not None:
        fl = torch.from_numpy(labels_field()).to(dev)
        gl = lower_star_grad(fl)
        gtl = 1e-6 * float(fl.abs().max())
        integ_l = dict(INTEG, gradient_threshold=gtl)
        plain_l = integrated_labels(fl, gl, **integ_l)
        learned_l = triage.triage_labels(fl, gl, net, **integ_l) if net is not None else None
        oproc, oq, opath = oracle_job
        oproc.join()
        t_oracle = oq.get() if oproc.exitcode == 0 else None
        if oproc.exitcode == 0:
            want = np.load(opath)
            mismatch = {"workload": "256^3 float32, 64 Gaussians + U[-1e-3,1e-3] noise, seed 0; error 1e-4, gradient "
                                    "threshold 1e-6 max|f|, 4000 iterations, 0.25 voxel",
                        "plain": {k: float((plain_l[k].cpu().numpy() != want[k]).mean()) for k in ("asc", "dsc")},
                        "oracle": "FP64 single-thread restatement, equal to the reference at one thread",
                        "oracle_seconds": t_oracle}
            if learned_l is not None:
                mismatch["learned"] = {k: float((learned_l[k].cpu().numpy() != want[k]).mean()) for k in ("asc", "dsc")}
            if NOISE_FILE.exists():
                nz = json.loads(NOISE_FILE.read_text())
                mismatch["reference_own_variation"] = {
                    "what": f"the reference at {nz['threads']} threads vs one thread, largest of {nz['runs']} runs",
                    **{k: nz["fields"]["gauss256_cfg2"][k] for k in ("asc", "dsc")}}
            os.unlink(opath)
        del fl, gl, plain_l, learned_l

    if rank == 0:
        mode = ".grad only" if args.grad_only else (
            ".grad + learned-triage labels" if step_net is not None else ".grad + plain integrated labels")
        wl = f"{mode}, {wl_name}, seed = rank"
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32" if args.grad_only else "f32+f64", "data": "synthetic",
                "config": {"workload": wl,
                           "vertices": V, "cells": C, "parallelism": f"replicas x{ws}",
                           "labels": "error 1e-4, gradient threshold 1e-6 max|f|, 4000 iterations, 0.25 voxel",
                           "l2": f"inputs larger than L2 (f {4 * V >> 20} MiB, .grad {C >> 20} MiB); no flush"},
                "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                        "ms_per_step": t_e2e * 1e3, "ms_calls": [round(t, 1) for t in e2e_ms], "api": api},
                "grad": {"value": V / (t_grad * 1e-3) / 1e9, "unit": UNIT, "ms_per_step": t_grad},
                "roofline": roofline,
                "kernels": kernels,
                "gpu_launches": launches,
                "clocks": clocks}
        line.update(line_extra)
        if grad_2d is not None:
            line["grad_2d"] = grad_2d
        if graph is not None:
            line["ms_graph"] = graph
        if conform is not None:
            line["conforming_grad"] = conform
        if mismatch is not None:
            line["mismatch_vs_fp64_oracle"] = mismatch
        if batch is not None:
            line["batch"] = batch
        if ws == 1 and not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline(f_np, grad_only=args.grad_only)
        print(json.dumps(line), flush=True)
    if pg is not None:
        pg.destroy_process_group()


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per launch from one ncu
# --set full capture of each kernel at 256^3 (f and .grad together 201 MB, above the
# L2), scaled to 512^3 by the vertex count (x 8): the traffic grows with the volume.
# ldir_stage = tile + check kernels (the walk is below 5% of the stage's time).
_T_LSTAR = 67.342e6 + 78.792e6
_T_LDIR = 133.928e6 + 96.585e6 + 147.920e6 + 9.383e6
TRAFFIC_PER_LAUNCH: dict = {
    ("lstar_kernel", 256): _T_LSTAR,
    ("ldir_stage", 256): _T_LDIR,
    ("lstar_kernel", 512): _T_LSTAR * 8,
    ("ldir_stage", 512): _T_LDIR * 8,
}
# Warp instructions per unit from the same captures (smsp__inst_executed.sum): the .grad
# kernels are integer-issue bound, so their ceiling is the SMs' issue rate (152 SMs x 4
# schedulers x clock), not HBM.  lstar_kernel: 1.320 G per 256^3 launch (per vertex);
# ldir stage: tile 1.806 G + check 0.111 G per 256^3 (per cell).
WARP_INST_PER_UNIT: dict = {
    "lstar_kernel": (1.320036e9 / 256 ** 3, "vertex"),
    "ldir_stage": ((1.805696e9 + 0.110793e9) / 511 ** 3, "cell"),
}
SCHEDULERS_PER_SM = 4
SMS = 152

# FP32 operations of one adaptive-Euler iteration as the reference's advector states
# it: two trilinear interpolations in the (1 - t) a + t b form (2 x 73), |g| (6), the
# step clamp (2), the full and two half steps with the error test and the move (29).
# The kernels execute fewer (each voxel's x-differences are taken once at entry); the
# count is the algorithmic work, the same for every implementation.
FLOP_PER_ITERATION = 183
FP32_LANES_PER_SM = 128
SM_MAX_MHZ = 2070


def main():
    args = parse_args()
    ws, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, ws, rank)
    else:
        run_ours(args, ws, rank, local)


if __name__ == "__main__":
    main()
