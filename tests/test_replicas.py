"""Multi-GPU path = independent replicas: the host-side logic of bench.py (per-rank seeds, the barrier, the
maximum of the timed totals over the ranks, the whole-job rate) run as two gloo ranks on the CPU."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, w, lr = bench.dist_info()
        local_total = 1.5 + rank            # each replica's timed total (s): rank 1 is the slower one
        dist.barrier()
        slowest = bench.max_over_ranks(local_total, w, "cpu")
        out[rank] = (r, w, lr, bench.replica_seed(r), slowest, bench.aggregate_rate(w, 5, slowest))
    finally:
        dist.destroy_process_group()


def test_two_replicas_with_gloo():
    world = 2
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank_main, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert sorted(res) == [0, 1]
    seeds = {res[r][3] for r in res}
    assert len(seeds) == 2                        # independent design loops
    for r, (rank, w, lr, seed, slowest, rate) in res.items():
        assert (rank, w, lr) == (r, 2, r)
        assert slowest == pytest.approx(2.5)      # the max over the ranks, on every rank
        assert rate == pytest.approx(2 * 5 / 2.5)  # whole-job design iterations per second


def test_single_rank_needs_no_collective():
    import bench
    assert bench.max_over_ranks(3.0, 1, "cpu") == 3.0
    assert bench.aggregate_rate(1, 4, 2.0) == 2.0
