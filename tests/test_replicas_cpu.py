"""The multi-GPU form of the path is replicas only: every rank labels its own volume,
no data moves between ranks, and the whole-job throughput is the sum of the volumes
over the slowest rank's time.  The host-side logic of that (bench.py's max over ranks,
the aggregate, the reference arm running on rank 0 alone) runs here on CPU ranks over
gloo, world size 2."""
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, ws, port, out_dir):
    import torch.distributed as dist
    sys.path.insert(0, str(ROOT))
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    assert bench.dist_setup() == (ws, rank, rank)
    # rank r's replica took (r + 1) * 100 ms: the job is as fast as the slowest rank
    t = bench.max_over_ranks((rank + 1) * 0.1, dist, "cpu")
    v = bench.aggregate_gvps(ws, 512 ** 3, t)
    dist.barrier()
    dist.destroy_process_group()
    Path(out_dir, f"r{rank}.txt").write_text(f"{t} {v}")


def test_replicas_max_over_ranks_and_aggregate(tmp_path):
    import torch.multiprocessing as mp
    ws = 2
    mp.start_processes(_rank_main, args=(ws, _free_port(), str(tmp_path)), nprocs=ws, join=True, start_method="spawn")
    vals = [tuple(map(float, (tmp_path / f"r{r}.txt").read_text().split())) for r in range(ws)]
    for t, v in vals:
        assert t == pytest.approx(0.2)
        assert v == pytest.approx(2 * 512 ** 3 / 0.2 / 1e9)


def test_reference_arm_runs_on_rank_zero_only(capsys, monkeypatch):
    sys.path.insert(0, str(ROOT))
    import bench
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0"])
    args = bench.parse_args()
    assert bench.run_reference(args, 2, 1) is None  # rank 1: no work, no output
    assert capsys.readouterr().out == ""
