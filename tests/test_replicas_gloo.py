"""Multi-GPU form: replicas only.  Independent simulations are sharded over
ranks with no data-path collective; the only collectives are the bench's
barrier and max-over-ranks time.  Two gloo ranks on the CPU run their shares
of a small ensemble on the oracle and check the partition and the reduction."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    sys.path.insert(0, os.path.join(root, "swalbe.jl_gb300"))
    import oracle
    from swalbe_gb300 import configs
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    members = list(range(6))
    mine = configs.shard(members, rank, world)
    masses = {}
    for i in mine:  # each member: a small film, its own seed
        P = oracle.params(24 + 4 * i, 20)
        h0 = 1.0 + 0.05 * np.random.default_rng(i).uniform(-1, 1, (24 + 4 * i, 20))
        r = oracle.FusedState(P, h0).run(30)
        masses[i] = float(r.height.sum())
    gathered = [None] * world
    dist.all_gather_object(gathered, masses)
    t = torch.tensor([float(rank + 1)])
    dist.all_reduce(t, op=dist.ReduceOp.MAX)  # the bench's max-over-ranks time
    dist.barrier()
    if rank == 0:
        q.put((gathered, float(t.item())))
    dist.destroy_process_group()


def test_two_rank_replicas_partition_and_reduce():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    gathered, tmax = q.get(timeout=240)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    keys = [k for g in gathered for k in g]
    assert sorted(keys) == list(range(6)) and len(set(keys)) == 6  # disjoint, complete
    assert tmax == 2.0
    # each share's results equal a single-process run of the same members
    import oracle
    for g in gathered:
        for i, m in g.items():
            P = oracle.params(24 + 4 * i, 20)
            h0 = 1.0 + 0.05 * np.random.default_rng(i).uniform(-1, 1, (24 + 4 * i, 20))
            assert m == float(oracle.FusedState(P, h0).run(30).height.sum())
