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


def _stats_rank(rank, world, port, out_dir):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from coarseair_gb300 import api, build, systems
    import test_stats_host as T
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    items, rows, runs = T._ring_rows_two_runs()
    P = T._params(3, (1, 0, 0, 0, 0), T._xmu(systems.n3_config().masses))
    items_pass, counts_pass = T.numpy_passes(build.LIB, P, 3)
    sel = (rows["item"] == 1) | (np.arange(len(rows)) % 2 == 0) if rank == 0 else \
        (rows["item"] != 1) & (np.arange(len(rows)) % 2 == 1)
    lines = api.replica_statistics(P, items, rows[sel], runs, items_pass, counts_pass)
    np.save(os.path.join(out_dir, "stats%d.npy" % rank), lines)
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_exchange_only_statistics_sums(tmp_path, gpu_lib, oracle_lib):
    """The multi-GPU statistics path on two gloo ranks: each rank holds half of the rows (one rank all of
    an item's), the ranks exchange the summed totals and counts (api.replica_statistics), and both
    end with the lines of all rows together."""
    pytest.importorskip("torch")
    import torch.multiprocessing as tmp
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import test_stats_host as T
    from coarseair_gb300 import systems
    world, port = 2, _free_port()
    tmp.start_processes(_stats_rank, args=(world, port, str(tmp_path)), nprocs=world, join=True,
                        start_method="spawn")
    got = [np.load(tmp_path / ("stats%d.npy" % r)) for r in range(world)]
    items, rows, runs = T._ring_rows_two_runs()
    P = T._params(3, (1, 0, 0, 0, 0), T._xmu(systems.n3_config().masses))
    keep = (rows["status"] == 0) & (np.abs(rows["dH"]) <= P.ham_abs_tol)
    one = T._host_statistics(T._load(gpu_lib), P, items, rows, runs, keep, 3)
    assert np.array_equal(got[0], got[1]) and np.array_equal(got[0], one)
