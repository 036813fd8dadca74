"""The multi-GPU form of bench.py is replicas only: every rank runs the whole
workload and the job's time is the slowest rank's.  The timing reduction runs
here as two gloo ranks on CPU."""
import os
import sys
from pathlib import Path

import pytest

torch = pytest.importorskip("torch")
ROOT = Path(__file__).resolve().parents[1]


def _rank(rank, ws, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    sys.path.insert(0, str(ROOT))
    import bench
    t = bench.max_over_ranks(10.0 + 5.0 * rank, ws)
    bench.barrier(ws)
    out.put((rank, t))
    dist.destroy_process_group()


def test_max_over_ranks_gloo_world_size_2():
    import socket
    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == {0: 15.0, 1: 15.0}
