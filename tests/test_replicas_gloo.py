"""Multi-process host logic of bench.py's replica runs (one process per GPU, weak
scaling, no data-path collective), on CPU with the gloo backend at world size 2:
process-group set-up from the torchrun environment, the barrier, the max over ranks
of the timed region, and that only rank 0 runs the CPU reference arm."""
import io
import os
import socket
import sys
from argparse import Namespace
from contextlib import redirect_stdout

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    args = Namespace(impl="reference", steps=1, warmup=0, cpu_n=8)
    r, w = bench.dist_init(args)
    assert (r, w) == (rank, world)
    assert dist.get_backend() == "gloo"
    bench.barrier(w)
    # each rank's timed region; the job's time is the slowest rank's
    m = bench.max_over_ranks(1.5 * (rank + 1), w)
    buf = io.StringIO()
    rc = None
    if rank != 0:
        with redirect_stdout(buf):
            rc = bench.run_reference(args, r, w)
    bench.barrier(w)
    with open(os.path.join(out_dir, f"rank{rank}.txt"), "w") as f:
        f.write(f"{m} {rc} {len(buf.getvalue())}\n")
    dist.destroy_process_group()


def test_replicas_two_ranks_gloo(tmp_path):
    world = 2
    mp.spawn(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    rows = [open(tmp_path / f"rank{r}.txt").read().split() for r in range(world)]
    # both ranks see the maximum of {1.5, 3.0}
    assert [float(x[0]) for x in rows] == [3.0, 3.0]
    # rank 1 leaves the reference arm at once, printing nothing
    assert rows[1][1] == "0" and rows[1][2] == "0"


def test_single_process_needs_no_process_group(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.delenv("WORLD_SIZE", raising=False)
    monkeypatch.delenv("RANK", raising=False)
    assert bench.dist_init(Namespace(impl="ours")) == (0, 1)
    assert bench.max_over_ranks(2.5, 1) == 2.5
    bench.barrier(1)
