"""The multi-GPU path of the benchmark on CPU: replicas, one text per rank.

A single text does not shard (the dictionary dedup and the parse suffix
array are global), so N GPUs run N independent replicas; the only exchange
is the max over ranks of the step times.  Two gloo ranks on CPU check that
reduction and the job throughput derived from it.
"""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist              # noqa: E402
import torch.multiprocessing as mp            # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, out):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        ms, e2e, v, ve = bench.replica_timing(10.0 + rank, 20.0 + 3 * rank, ws, 1_000_000, "cpu")
        out.put((rank, ms, e2e, v, ve))
    finally:
        dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank():
    ws = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, ws, port, q)) for r in range(ws)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(ws))
    for rank, ms, e2e, v, ve in res:
        assert ms == 11.0 and e2e == 23.0              # max over the two ranks
        assert v == pytest.approx(ws * 1_000_000 / 0.011 / 1e6)
        assert ve == pytest.approx(ws * 1_000_000 / 0.023 / 1e6)


def test_one_rank_needs_no_process_group():
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    assert bench.replica_timing(4.0, 8.0, 1, 2_000_000, "cpu") == (4.0, 8.0, 500.0, 250.0)

