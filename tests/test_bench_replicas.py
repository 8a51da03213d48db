"""The N-GPU bench path is N independent replicas (the path does not shard): each rank times
its own copy of the workload between host barriers, rank 0 prints the slowest rank's time,
and the reference arm runs on rank 0 only. These are its host pieces, as two gloo ranks on the
CPU (no GPU)."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        assert bench.dist_info() == (ws, rank, rank)
        bench.replica_barrier(ws)
        m = bench.replica_max(1.5 + rank, ws)
        # the reference arm: rank 0 alone runs; the others return at once without work
        ref = None
        if rank != 0:
            ref = bench.run_reference(None)
        out.put((rank, m, ref))
        bench.replica_barrier(ws)
    finally:
        dist.destroy_process_group()


def test_two_replicas_take_the_slowest_rank():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    ws, port = 2, _free_port()
    out = mp.Queue()
    procs = [mp.Process(target=_rank, args=(r, ws, port, out)) for r in range(ws)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    res = sorted(out.get(timeout=5) for _ in range(ws))
    assert [m for _, m, _ in res] == [2.5, 2.5]
    assert res[1][2] is None
