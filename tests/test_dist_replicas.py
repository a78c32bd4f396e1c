"""Multi-GPU path of bench.py: independent replicas, max-over-ranks timing (gloo, CPU)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, ws, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    import bench
    bench.dist_barrier(ws)
    seconds = 1.0 + rank          # rank 1 is the slow replica
    v = bench.replica_throughput(10, seconds, ws)
    out[rank] = (bench.dist_max(float(rank), ws), v)
    dist.destroy_process_group()


def test_two_replicas_report_whole_job_throughput():
    ws = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        procs = [ctx.Process(target=_worker, args=(r, ws, port, out)) for r in range(ws)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        for r in range(ws):
            mx, v = out[r]
            assert mx == 1.0                 # max over ranks
            assert abs(v - 2 * 10 / 2.0) < 1e-12   # 20 units over the slowest rank's 2 s
