"""Two ranks on CPU (gloo): disjoint k-ranges of one mesh, partial sums
reduced with one all_reduce, equal to the single-process Hall conductivity.
The per-range sums come from the oracle (no GPU here); the sharding and the
reduction are the library's (rustb_gb300.shard)."""

import os
import socket

import numpy as np
import torch.distributed as dist
import torch.multiprocessing as mp

from rustb_gb300 import shard


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    import torch

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    import models as M
    from oracle import tb_oracle as O

    h = M.haldane()
    mesh = (12, 10)
    nk = 120
    k = O.gen_kmesh(mesh)
    mus = np.array([-0.5, 0.0, 0.5])
    part = np.zeros(len(mus))
    for k0, cnt in shard.rank_ranges(nk, world, rank, 16):
        Om, E = O.berry_on(h, k[k0:k0 + cnt], np.eye(2))
        for j, mu in enumerate(mus):
            part[j] += (Om * O.fermi(E, mu, 0.0)).sum()
    t = torch.tensor(part, dtype=torch.float64)
    dist.all_reduce(t)
    if rank == 0:
        q.put(t.numpy() / nk / float(np.linalg.det(h.lat)))
    dist.destroy_process_group()


def test_two_rank_k_shards_equal_single_process():
    import sys
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    import models as M
    from oracle import tb_oracle as O

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    ref = O.hall_conductivity(M.haldane(), (12, 10), np.eye(2), np.array([-0.5, 0.0, 0.5]))
    assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(ref))


def test_ranges_cover_mesh_once():
    nk, world, batch = 1000, 3, 64
    seen = np.zeros(nk, dtype=int)
    for r in range(world):
        for k0, cnt in shard.rank_ranges(nk, world, r, batch):
            seen[k0:k0 + cnt] += 1
    assert np.all(seen == 1)
    assert shard.step_range(100, 30, 2, 1, 1) == (90, 10)
