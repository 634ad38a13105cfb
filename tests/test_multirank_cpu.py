"""World-size-2 checks of the bench's multi-rank host logic on CPU (gloo): each rank runs an
independent replica of the workload (no collective on the data path), the timing is the max
over ranks, and the reported throughput aggregates every rank's interactions."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, ws, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        got_ws, got_rank, got_local = bench.dist_env()
        ms = 10.0 + 5.0 * rank                       # rank 1 is the slow one
        slowest = bench.max_over_ranks(ms)
        rate = bench.aggregate_rate(1e12, got_ws, slowest)
        x, _, _, s = bench.make_workload(bench.SEED + got_rank, 2048)
        out[rank] = (got_ws, got_rank, got_local, slowest, rate, float(x[0]), float(s.sum()))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_ranks_max_time_and_aggregate_rate():
    ws = 2
    with mp.get_context("spawn").Manager() as m:         # no fork of this multi-threaded process
        out = m.dict()
        mp.start_processes(_rank_main, args=(ws, _free_port(), out), nprocs=ws, join=True, start_method="spawn")
        res = dict(out)
    assert sorted(res) == [0, 1]
    for rank, (gws, grank, glocal, slowest, rate, x0, ssum) in res.items():
        assert (gws, grank, glocal) == (2, rank, rank)
        assert slowest == 15.0                        # the max over ranks, on every rank
        assert rate == pytest.approx(2 * 1e12 / 15e-3 / 1e9)
        assert abs(ssum - 1.0) < 1e-5
    assert res[0][5] != res[1][5]                     # independent replicas: different seeds


def test_single_process_helpers():
    import bench
    assert bench.max_over_ranks(3.5) == 3.5
    assert bench.aggregate_rate(1e12, 1, 250.0) == pytest.approx(4000.0)
    assert np.isclose(bench.aggregate_rate(2e9, 4, 1.0), 8000.0)
