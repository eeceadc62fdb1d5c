"""Multi-process (gloo, world_size 2) check of the sharded batch: each rank
steps its share of the worlds with the CPU oracle and the gathered per-world
hashes equal a single-process run; no simulation data crosses ranks."""
import os
import socket

import numpy as np
import torch.distributed as dist
import torch.multiprocessing as mp

from fallingsand3d_gb300 import sharding


def _worlds(fs3d, n):
    dims, seeds = fs3d.gen_batch_dims(11, n)
    return [(tuple(int(min(v, 32)) for v in dims[w]), int(seeds[w])) for w in range(n)]


def _run(worlds, idx, steps):
    import oracle_lib
    import fallingsand3d_gb300 as fs3d
    orc = oracle_lib.load()
    out = {}
    for i in idx:
        (X, Y, Z), seed = worlds[i]
        g = fs3d.gen_batch_world(seed, X, Y, Z)
        orc.run(g, seed, 0, steps, nthreads=1)
        out[i] = orc.hash(g)
    return out


def _worker(rank, size, port, q):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=size)
    import fallingsand3d_gb300 as fs3d
    worlds = _worlds(fs3d, 10)
    parts = sharding.strong_split(worlds, size)
    mine = _run(worlds, parts[rank], 6)
    gathered = [None] * size
    dist.all_gather_object(gathered, mine)
    if rank == 0:
        merged = {}
        for g in gathered:
            merged.update(g)
        q.put(merged)
    dist.destroy_process_group()


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def test_strong_split_balances_and_covers(fs3d):
    worlds = _worlds(fs3d, 50)
    parts = sharding.strong_split(worlds, 4)
    assert sorted(i for p in parts for i in p) == list(range(50))
    loads = [sum(np.prod(worlds[i][0]) for i in p) for p in parts]
    assert max(loads) - min(loads) <= max(np.prod(w[0]) for w in worlds)
    assert sharding.weak_master(5, 3) == 8


def test_two_rank_gloo_matches_single_process(fs3d):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    merged = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    worlds = _worlds(fs3d, 10)
    assert merged == _run(worlds, range(10), 6)
