"""Multi-rank path on CPU: two gloo ranks take disjoint, cost-balanced shards
of independent sector solves and gather the results; the union equals the
serial answers.  (GPU runs use one GPU per rank the same way.)"""
import os
import socket

import numpy as np
import torch.distributed as dist
import torch.multiprocessing as mp

from realspace_exactdiagonalization_gb300.sharding import shard, shard_indices


def test_shard_indices_partition_and_balance():
    costs = [5, 1, 1, 1, 3, 2, 2, 8, 1]
    parts = shard_indices(costs, 3)
    assert sorted(i for p in parts for i in p) == list(range(len(costs)))
    loads = [sum(costs[i] for i in p) for p in parts]
    assert max(loads) - min(loads) <= max(costs)
    assert shard_indices(costs, 3) == parts  # deterministic


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _solve(item):
    import oracle as O
    from cases import case_by_name, oracle_objects

    name, k = item
    _, sec, op = oracle_objects(O, case_by_name(name), k)
    return (name, k, float(np.linalg.eigvalsh(op.dense())[0]) if sec.dim else None)


ITEMS = [("checkerboard3x2_f_flux", k) for k in range(6)] + [("haldane2x3", k) for k in range(6)]


def _worker(rank, world, port, out):
    import sys

    here = os.path.dirname(os.path.abspath(__file__))
    sys.path[:0] = [here, os.path.join(os.path.dirname(here), "oracle"), os.path.dirname(here)]
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = shard(ITEMS, rank, world, cost=lambda it: 2.0 if it[0].startswith("checker") else 1.0)
    res = [_solve(it) for it in mine]
    gathered = [None] * world
    dist.all_gather_object(gathered, res)
    if rank == 0:
        out.put([r for part in gathered for r in part])
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_cover_all_items():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = q.get(timeout=240)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    serial = [_solve(it) for it in ITEMS]
    assert sorted(got, key=lambda t: (t[0], t[1])) == sorted(serial, key=lambda t: (t[0], t[1]))
