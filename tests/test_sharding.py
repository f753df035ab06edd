"""Box sharding over ranks: the partition and the host-side gather, run as
two gloo ranks on the CPU (each rank evaluates its boxes with the oracle)."""
import os

import numpy as np
import pytest
import torch.multiprocessing as mp

from macsimus_gb300 import sharding


def test_partition_balances_and_covers():
    rng = np.random.default_rng(3)
    costs = list(rng.uniform(1, 100, 57))
    for n in (1, 2, 3, 8):
        parts = sharding.partition(costs, n)
        assert sorted(i for p in parts for i in p) == list(range(57))
        loads = [sum(costs[i] for i in p) for p in parts]
        # LPT is within 4/3 of the optimum; the mean is a lower bound of it
        assert max(loads) <= 4.0 / 3.0 * max(np.mean(loads), max(costs)) + 1e-9
    assert sharding.partition([5, 5, 5, 5], 2) == sharding.partition([5, 5, 5, 5], 2)


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from macsimus_gb300 import configs
    from oracle import oracle as O
    boxes = configs.ionic_boxes(6, seed=21, nmin=100, nmax=300)
    costs = [sharding.box_cost(b["system"].ns, len(O.kvectors([b["L"]] * 3, b["kappa"])[0]),
                               b["cutoff"], b["L"]) for b in boxes]
    mine = sharding.partition(costs, world)[rank]
    local = {}
    for i in mine:
        b = boxes[i]
        orc = O.Oracle(b["system"], [b["L"]] * 3, b["cutoff"], b["alpha"], b["kappa"])
        _, en = orc.forces(b["r"], nthreads=1)
        local[i] = en["el"] + en["lj"]
    merged = sharding.gather_results(local, rank, world)
    if rank == 0:
        q.put(merged)
    dist.destroy_process_group()


def test_two_rank_gather_matches_serial():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    merged = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    from macsimus_gb300 import configs
    from oracle import oracle as O
    boxes = configs.ionic_boxes(6, seed=21, nmin=100, nmax=300)
    assert sorted(merged) == list(range(6))
    for i, b in enumerate(boxes):
        orc = O.Oracle(b["system"], [b["L"]] * 3, b["cutoff"], b["alpha"], b["kappa"])
        _, en = orc.forces(b["r"], nthreads=1)
        assert merged[i] == en["el"] + en["lj"]
