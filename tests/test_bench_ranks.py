"""bench.py's multi-rank logic on CPU: two gloo ranks (127.0.0.1) agree on the
max-over-ranks time, pass the barrier, and the reference arm prints only on
rank 0 (the other rank exits 0 without work)."""
import io
import json
import os
import socket
import sys
from contextlib import redirect_stdout

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    t = bench._max_over_ranks(1.0 + rank, world)
    bench._barrier(world)
    args = type("A", (), {"warmup": 0, "steps": 1, "gpus": world})()
    buf = io.StringIO()
    if rank != 0:
        with redirect_stdout(buf):
            rc = bench.run_reference(args)
    else:
        rc = 0
    with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
        json.dump({"max": t, "rc": rc, "printed": buf.getvalue()}, f)
    dist.destroy_process_group()


def test_two_gloo_ranks(tmp_path):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    r0 = json.load(open(tmp_path / "rank0.json"))
    r1 = json.load(open(tmp_path / "rank1.json"))
    assert r0["max"] == r1["max"] == 2.0
    assert r1["rc"] == 0 and r1["printed"] == ""
