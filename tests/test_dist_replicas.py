"""The N>1 host path on CPU: two gloo ranks take their share of independent
gridding units (channels), grid them with the oracle, and together reproduce
the single-process result; the step-time reduction returns the max."""
import os
import socket

import numpy as np


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _units(n_units=5, n=300, G=64, seed=0):
    rng = np.random.default_rng(seed)
    out = []
    for u in range(n_units):
        m = n * (u + 1)
        uvw = np.column_stack([rng.uniform(-20, 20, m), rng.uniform(-20, 20, m), np.zeros(m)])
        vis = rng.standard_normal(m) + 1j * rng.standard_normal(m)
        out.append((uvw, vis))
    sup = np.array([6], np.int32)
    gcf = rng.standard_normal(64 * 36) + 1j * rng.standard_normal(64 * 36)
    return out, sup, gcf, G


def _grid_unit(unit, sup, gcf, G):
    from oracle import oracle as O

    uvw, vis = unit
    g = np.zeros((G, G), np.complex128)
    O.scatter_planes(1.0, G, 6, uvw, vis, np.zeros(len(vis), np.int32), sup, gcf,
                     np.array([0], np.int64), g)
    return g


def _worker(rank, world, port, q):
    import torch
    import torch.distributed as dist

    from rc_gb300.shard import max_over_ranks, my_units

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    units, sup, gcf, G = _units()
    costs = [len(u[1]) for u in units]
    mine = my_units(costs, world, rank)
    grids = {u: _grid_unit(units[u], sup, gcf, G) for u in mine}
    gathered = [None] * world
    dist.all_gather_object(gathered, grids)
    t = max_over_ranks(1.0 + rank)
    if rank == 0:
        merged = {}
        for d in gathered:
            merged.update(d)
        q.put((sorted(merged), {k: v.tobytes() for k, v in merged.items()}, t))
    dist.barrier()
    dist.destroy_process_group()


def test_partition_is_balanced_and_complete():
    from rc_gb300.shard import partition

    costs = [9, 1, 8, 2, 7, 3, 6, 4, 5]
    parts = partition(costs, 3)
    assert sorted(sum(parts, [])) == list(range(9))
    loads = [sum(costs[i] for i in p) for p in parts]
    # the greedy bound: no rank exceeds the mean by more than one unit's cost
    assert max(loads) <= sum(costs) / 3 + max(costs)
    assert max(loads) <= 16


def test_two_gloo_ranks_reproduce_single_process():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    keys, blobs, tmax = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    units, sup, gcf, G = _units()
    assert keys == list(range(len(units)))
    for k in keys:
        got = np.frombuffer(blobs[k], np.complex128).reshape(G, G)
        assert np.array_equal(got, _grid_unit(units[k], sup, gcf, G))
    assert tmax == 2.0
