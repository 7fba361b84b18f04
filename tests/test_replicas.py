"""The multi-GPU bookkeeping (flowfpmpp_gb300.replicas) with two gloo ranks on
the CPU: barriers, the max-reduction of the time and the job throughput the
benchmark reports (world x units / slowest rank's time)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    from flowfpmpp_gb300.replicas import Replicas
    r = Replicas(world=world, rank=rank)
    r.barrier()
    value, t = r.throughput(units_per_rank=10.0, seconds=1.0 + rank)  # rank 1 is the slow one
    m = r.max(rank * 3.5)
    r.barrier()
    r.close()
    with open(os.path.join(out, f"rank{rank}.txt"), "w") as fh:
        fh.write(f"{value} {t} {m}\n")


def test_two_replicas(tmp_path):
    import torch.multiprocessing as mp
    world = 2
    mp.spawn(_rank, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    for rank in range(world):
        value, t, m = (float(x) for x in (tmp_path / f"rank{rank}.txt").read_text().split())
        assert t == 2.0 and value == pytest.approx(world * 10.0 / 2.0) and m == 3.5


def test_one_replica():
    from flowfpmpp_gb300.replicas import Replicas
    r = Replicas(world=1, rank=0)
    assert r.throughput(4.0, 2.0) == (2.0, 2.0) and r.max(7.0) == 7.0
    r.barrier()
    r.close()
