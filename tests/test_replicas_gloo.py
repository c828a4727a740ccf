"""The N > 1 path of bench.py on the CPU: `--gpus N` runs N independent replicas
of the workload (one rank per GPU, no data-path collective); the step time is the
slowest rank's, taken by one MAX all-reduce, and only rank 0 prints.  Two gloo
ranks check that reduction and the rank bookkeeping (no GPU needed)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, out):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(ws), "LOCAL_RANK": str(rank)})
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        w, r, local = bench._dist()
        ms = bench.replica_max_ms(10.0 + 5.0 * rank, w, "cpu")
        out[rank] = (w, r, local, ms)
    finally:
        dist.destroy_process_group()


def test_replicas_take_the_slowest_rank_time():
    ws = 2
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(ws, port, out), nprocs=ws, join=True)
        res = dict(out)
    assert sorted(res) == [0, 1]
    for rank, (w, r, local, ms) in res.items():
        assert (w, r, local) == (ws, rank, rank)
        assert ms == 15.0  # both ranks see the slowest replica's time


def test_single_process_needs_no_collective():
    import bench

    assert bench.replica_max_ms(12.5, 1, "cpu") == 12.5
