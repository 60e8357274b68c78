"""The multi-process path of bench.py on CPU: two gloo ranks (127.0.0.1) run
replica_throughput with different local times; both get the slowest rank's time
and the whole-job throughput (units of both ranks over that time)."""

import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, port, out):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE="2", RANK=str(rank),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=2)
    try:
        ms, ups = bench.replica_throughput([10.0, 25.0][rank], 1.0e9, device="cpu")
        dist.barrier()
        with open(os.path.join(out, f"r{rank}.txt"), "w") as f:
            f.write(f"{ms} {ups}")
    finally:
        dist.destroy_process_group()


def test_replica_throughput_two_gloo_ranks(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    if not torch.distributed.is_available():
        pytest.skip("torch.distributed not available")
    mp.spawn(_rank, args=(_free_port(), str(tmp_path)), nprocs=2, join=True)
    for r in range(2):
        ms, ups = map(float, open(tmp_path / f"r{r}.txt").read().split())
        assert ms == 25.0
        assert ups == pytest.approx(2.0e9 / 0.025)


def test_replica_throughput_single_process(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench

    monkeypatch.setenv("WORLD_SIZE", "1")
    ms, ups = bench.replica_throughput(20.0, 5.0e8)
    assert ms == 20.0 and ups == pytest.approx(2.5e10)
