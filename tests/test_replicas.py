"""The multi-GPU path is replicas only: trajectories are independent and shard by work item with no
exchange (each replica runs its own random-number streams, as the reference's processes do with
iProc), and the job time is the slowest replica's.  This covers that host logic with two gloo ranks
on the CPU: disjoint streams across ranks, the max-over-ranks reduction and the whole-job rate."""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import torch
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    res = {}
    for system in ("n3", "o3", "o4"):
        table, items = bench.SYSTEMS[system]["workload"](3000, rank)
        seeds = torch.tensor(items["seed"].astype(np.int64))
        gathered = [torch.zeros_like(seeds) for _ in range(world)]
        dist.all_gather(gathered, seeds)
        res[system] = [g.numpy() for g in gathered]
        res[system + "_ntraj"] = int(items["ntraj"].sum())
    ms = 1000.0 + 250.0 * rank            # a slower second replica
    res["ms_max"] = bench.max_over_ranks(ms, dist, torch.tensor([0.0]))
    res["rate"] = bench.aggregate_rate(3000, 2, world, res["ms_max"])
    np.save(os.path.join(out_dir, "rank%d.npy" % rank), res, allow_pickle=True)
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_draw_disjoint_streams_and_report_the_slowest(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as tmp
    world, port = 2, _free_port()
    tmp.start_processes(_rank_main, args=(world, port, str(tmp_path)), nprocs=world, join=True,
                        start_method="spawn")
    outs = [np.load(tmp_path / ("rank%d.npy" % r), allow_pickle=True).item() for r in range(world)]
    for system in ("n3", "o3", "o4"):
        a, b = outs[0][system]
        assert np.array_equal(outs[1][system][0], a)        # every rank sees the same gather
        assert len(np.intersect1d(a, b)) == 0              # no stream repeated across replicas
        assert outs[0][system + "_ntraj"] == 3000
    for o in outs:
        assert o["ms_max"] == 1250.0
        assert o["rate"] == pytest.approx(3000 * 2 * world / 1.25)
