"""Multi-rank host logic on CPU (gloo, world_size 2): systems are spread over ranks by cost with
no data-path collective, and the per-system results come back to every rank."""
import os
import socket

import numpy as np
import pytest

from quack_gb300 import shard, synth


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        systems = synth.batch_systems(16, 24, 64, seed=1)
        costs = [shard.cost(s["N"], s["nO"]) for s in systems]
        mine = shard.partition(costs, world)[rank]
        # stand-in for the per-system GPU result: a deterministic function of the system
        vals = [[s["N"], float(np.sum(s["eHF"]))] for s in (systems[i] for i in mine)]
        full = shard.gather(mine, vals, len(systems))
        q.put((rank, mine, full.tolist()))
    finally:
        dist.destroy_process_group()


def test_partition_covers_and_balances():
    systems = synth.batch_systems(256, 24, 160, seed=1)
    costs = [shard.cost(s["N"], s["nO"]) for s in systems]
    for world in (1, 2, 4, 8):
        shares = shard.partition(costs, world)
        flat = sorted(i for s in shares for i in s)
        assert flat == list(range(len(systems)))
        loads = [sum(costs[i] for i in s) for s in shares]
        # greedy LPT: no rank above the mean by more than the largest single system
        assert max(loads) - sum(loads) / world <= max(costs) + 1e-9


def test_gather_over_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = [q.get(timeout=120) for _ in range(2)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    systems = synth.batch_systems(16, 24, 64, seed=1)
    expect = np.array([[s["N"], float(np.sum(s["eHF"]))] for s in systems])
    mines = []
    for rank, mine, full in got:
        assert np.allclose(np.array(full), expect)
        mines.append(set(mine))
    assert not (mines[0] & mines[1]) and len(mines[0] | mines[1]) == len(systems)
