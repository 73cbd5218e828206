"""The multi-rank path of bench.py on the CPU: world size 2 over gloo.

The filters shard by stack with no exchange step ("replicas only"): each
rank filters its own stack; the job time is the maximum over ranks and the
throughput all ranks' voxels over it.  Ranks other than 0 of the reference
arm exit without work."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

from conftest import ROOT


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, ws, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import torch.distributed as tdist

    import bench
    tdist.init_process_group("gloo", rank=rank, world_size=ws)
    # rank r took 10 * (r + 1) ms for its 1e9 voxels
    ms, value = bench.replicas_value(10.0 * (rank + 1), 10**9, 1, ws)
    assert bench.dist()[:2] == (ws, rank)
    rc = bench.run_reference(type("A", (), {"steps": 1, "warmup": 1})()) if rank != 0 else None
    tdist.barrier()
    tdist.destroy_process_group()
    out[rank] = (ms, value, rc)


def test_max_over_ranks_and_aggregate_throughput():
    ws, port = 2, _free_port()
    with mp.get_context("spawn").Manager() as m:  # no fork of this (multi-threaded) process
        out = m.dict()
        mp.spawn(_rank, args=(ws, port, out), nprocs=ws, join=True)
        res = dict(out)
    for r in range(ws):
        ms, value, rc = res[r]
        assert ms == pytest.approx(20.0)                    # the slowest rank's time
        assert value == pytest.approx(2 * 1e9 / 20e-3 / 1e9)  # both ranks' voxels over it
    assert res[1][2] == 0                                   # the reference arm's other ranks do no work
