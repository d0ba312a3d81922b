"""The multi-replica bench path on CPU: two gloo ranks, each with its own step time, must agree on
the job's time (the slowest replica) and on the whole-job TEPS (replicas x edges x steps / time).
`python bench.py --gpus N` under torchrun runs the same functions over NCCL, one replica per GPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out):
    import sys
    sys.path.insert(0, ROOT)
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        local_ms = [40.0, 55.5][rank]
        dist.barrier()
        t = bench.max_over_ranks(local_ms, dist, "cpu")
        out[rank] = (t, bench.job_gteps(world, 16_499_362, 200, t))
    finally:
        dist.destroy_process_group()


def test_two_replicas_agree_on_time_and_teps():
    world = 2
    port = _free_port()
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert res[0] == res[1]
    t, gteps = res[0]
    assert t == 55.5
    assert abs(gteps - 2 * 16_499_362 * 200 / 55.5e-3 / 1e9) < 1e-9


def test_single_process_is_unchanged():
    import sys
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(12.5, None, "cpu") == 12.5
    assert bench.job_gteps(1, 1000, 10, 1.0) == pytest.approx(0.01)  # 10^4 edges in 1 ms
