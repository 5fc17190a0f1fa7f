"""The multi-GPU path of the bench runs N independent replicas; its only
collectives are the barrier and the maximum of the per-rank timings. Checked
here with two gloo ranks on the CPU."""
import os
import socket

import pytest

import replicas

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out_dir):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    dist.barrier()
    got = replicas.max_over_ranks([1.5 + rank, 10.0 - rank, 100.0 * (rank + 1)], dist)
    dist.barrier()
    dist.destroy_process_group()
    with open(os.path.join(out_dir, "rank%d.txt" % rank), "w") as f:
        f.write(repr(got))


def test_max_over_two_gloo_ranks(tmp_path):
    port = _free_port()
    torch.multiprocessing.spawn(_rank, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    for r in range(2):
        got = eval((tmp_path / ("rank%d.txt" % r)).read_text())
        assert got == [2.5, 10.0, 200.0]


def test_single_process_and_throughput():
    assert replicas.max_over_ranks([3.0, 4.0]) == [3.0, 4.0]
    # two replicas of a 1080p frame in 2 ms each: 2 * 2,073,600 rays / 2 ms
    assert abs(replicas.replica_throughput(2, 1920 * 1080, 2.0) - 2073.6) < 1e-9
