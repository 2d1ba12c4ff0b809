"""Host side of a multi-GPU batch (magnus_gb300.shard): cost-balanced
partition, and a world_size-2 gloo run on the CPU in which each rank
computes its share with the oracle and one gather returns every result in
instance order."""
import os
import socket

import numpy as np
import pytest

from magnus_gb300 import shard


def test_partition_covers_every_instance_once_and_balances():
    rng = np.random.default_rng(0)
    ds = rng.choice([2, 8, 32, 64, 128], size=200)
    Ss = rng.integers(257, 65537, size=200)
    ns = rng.integers(2, 7, size=200)
    costs = [shard.instance_cost(int(d), int(s), int(n)) for d, s, n in zip(ds, Ss, ns)]
    for world in (1, 2, 3, 8):
        parts = shard.partition(costs, world)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(200))
        loads = [sum(costs[i] for i in p) for p in parts]
        # greedy bound: no rank exceeds the mean by more than the largest item
        assert max(loads) <= sum(costs) / world + max(costs) + 1e-6


def test_partition_rejects_empty_world():
    with pytest.raises(ValueError):
        shard.partition([1.0], 0)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, specs, q):
    import sys
    import torch.distributed as dist
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, os.path.join(os.path.dirname(here), "oracle"))
    sys.path.insert(0, os.path.join(os.path.dirname(here), "magnus-dp_gb300"))
    import oracle as O
    from magnus_gb300 import shard as sh
    from magnus_gb300 import workloads
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        costs = [sh.instance_cost(d, S, n) for d, S, n in specs]

        def run(indices):
            out = {}
            for i in indices:
                d, S, n = specs[i]
                A = workloads.config0_samples(seed=i, d=d, samples=S)
                out[i] = (rank, O.forward(A, n, 0.0, 1.0, "sum", "Boole"))
            return out

        res = sh.sharded_map(run, costs, rank, world)
        q.put((rank, [(r, o.tolist()) for r, o in res]))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_shard_and_gather():
    import torch.multiprocessing as mp
    specs = [(2, 129, 3), (8, 65, 4), (4, 257, 2), (3, 33, 5), (2, 17, 2), (6, 129, 3)]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, specs, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    import oracle as O
    from magnus_gb300 import workloads
    costs = [shard.instance_cost(d, S, n) for d, S, n in specs]
    parts = shard.partition(costs, 2)
    for rank in (0, 1):
        assert len(got[rank]) == len(specs)  # every rank sees every result
        for i, (d, S, n) in enumerate(specs):
            owner, out = got[rank][i]
            assert i in parts[owner]  # computed by the rank the partition assigned
            ref = O.forward(workloads.config0_samples(seed=i, d=d, samples=S), n, 0.0, 1.0, "sum", "Boole")
            np.testing.assert_allclose(np.array(out), ref, rtol=0, atol=0)
