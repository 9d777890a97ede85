"""Replica aggregation of bench.py on two CPU ranks (gloo): every rank runs
its own catalogue, the job's step time is the slowest rank's and its
throughput counts the galaxies of all ranks.  The GPU runs use the same
function over NCCL (`bench.py --gpus N` under torchrun)."""

import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import importlib.util
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    # rank r: a step of (r + 1) ms over 1000 (r + 1) galaxies
    ms, n, v = bench.aggregate_replicas(float(rank + 1), 1000 * (rank + 1), world)
    out[rank] = (ms, n, v)
    dist.barrier()
    dist.destroy_process_group()


def test_aggregate_replicas_two_ranks():
    world = 2
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_rank, args=(world, _free_port(), out), nprocs=world, join=True)
        res = dict(out)
    for r in range(world):
        ms, n, v = res[r]
        assert ms == 2.0                      # the slowest rank
        assert n == 3000                      # all ranks' galaxies
        assert v == pytest.approx(3000 / 2e-3)


def test_aggregate_replicas_single():
    import importlib.util
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    assert bench.aggregate_replicas(4.0, 1000, 1) == (4.0, 1000, 1000 / 4e-3)
