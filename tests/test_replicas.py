"""The replica logic of bench.py on two CPU ranks (gloo): each rank runs an
independent system, the time is the max over ranks and the work the sum."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, ws, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    import sys
    from pathlib import Path
    sys.path.insert(0, str(Path(__file__).resolve().parent.parent))
    import bench
    got_ws, got_rank, _ = bench.dist_setup()
    assert (got_ws, got_rank) == (ws, rank)
    bench.barrier(ws)
    t = bench.allmax(ws, 1.0 + rank)            # rank-dependent "time"
    units = bench.allsum(ws, 100.0 * (rank + 1))
    out[rank] = (t, units)
    dist.destroy_process_group()


def test_two_rank_replicas_max_time_sum_work():
    ws = 2
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank_main, args=(ws, port, out), nprocs=ws, join=True)
        res = dict(out)
    assert res[0] == res[1] == (2.0, 300.0)
