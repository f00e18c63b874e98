"""Multi-GPU form of the path: independent replicas, one per rank, no
collective on the data path (the step does not shard).  These tests run the
host-side replica logic of bench.py as two gloo ranks on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

import bench  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        items = 1000 * (rank + 1)            # uneven replicas
        seconds = 2.0 if rank == 0 else 5.0  # rank 1 is the slowest
        rate, slowest = bench.aggregate_replicas(items, steps=4, seconds=seconds)
        out.put((rank, rate, slowest, bench.replica_seed("plain_small", rank)))
    finally:
        dist.destroy_process_group()


def test_replica_rate_is_all_items_over_slowest_rank():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, out)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(out.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    total_items = (1000 + 2000) * 4
    for rank, rate, slowest, seed in res:
        assert slowest == 5.0
        assert rate == pytest.approx(total_items / 5.0)
    assert res[0][3] != res[1][3], "replicas must be seeded differently"


def test_single_process_rate_is_local():
    rate, slowest = bench.aggregate_replicas(500, steps=2, seconds=0.5)
    assert (rate, slowest) == (2000.0, 0.5)


def test_reference_arm_prints_only_on_rank_zero(monkeypatch, capsys):
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")

    class Args:
        workload, steps, warmup, gpus, cpu_fraction = "plain_small", 1, 0, 2, 0.01
    bench.run_reference(Args())
    assert capsys.readouterr().out == ""
