"""The multi-GPU path of bench.py on the CPU: world size 2 over gloo.  The
solve does not shard (replicas only), so the one cross-rank operation is the
max over ranks of the step time; each rank also builds and skins nothing here
-- only the host-side logic is exercised."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, ws, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        w, r = bench._dist()
        assert (w, r) == (ws, rank)
        # every rank reports its own step time; all see the slowest one
        got = bench.reduce_max(10.0 + 5.0 * rank, w, device="cpu")
        out[rank] = got
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_reduce_max_two_ranks_gloo():
    import torch.multiprocessing as mp
    ws, port = 2, _free_port()
    with mp.get_context("spawn").Manager() as m:
        out = m.dict()
        mp.start_processes(_worker, args=(ws, port, out), nprocs=ws, start_method="spawn", join=True)
        assert dict(out) == {0: 15.0, 1: 15.0}


def test_reduce_max_single_rank():
    import bench
    assert bench.reduce_max(3.5, 1) == 3.5
