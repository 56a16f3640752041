"""Multi-rank shot sharding on CPU: two gloo ranks each migrate their block of
shots (with the oracle) and combine the stacks; the result equals a single
process stacking all shots."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from rtm_gpu_gb300.shard import combine_stacks, shard_shots


def test_shard_blocks_cover_shots_once():
    for n in (0, 1, 5, 64, 127):
        for w in (1, 2, 3, 8):
            got = [i for r in range(w) for i in shard_shots(n, r, w)]
            assert got == list(range(n))


def _problem():
    from util import small_problem
    return small_problem(NT=80, nz=30, nx=48, N2=6, M=4)


def _shots(p):
    return [(p.N2 + 1, p.N2 + x) for x in (4, 17, 30, 44)]


def _per_shot(p, shots, idx, seed=0):
    from oracle import oracle as orc
    ups, downs = [], []
    for i in idx:
        q = p.with_source(*shots[i])
        rng = np.random.default_rng(100 + i)
        seis = (rng.standard_normal((q.nrec, q.NT)) * 1e-2).astype(np.float32)
        r1, r2 = orc.migrate(q, seis)
        u, d = orc.finish_shot(q, r1, r2, 1e-4)
        ups.append(u.astype(np.float64))
        downs.append(d.astype(np.float64))
    return ups, downs


def _worker(rank, world, port, out):
    import sys
    sys.path.insert(0, os.path.dirname(__file__))
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    p = _problem()
    shots = _shots(p)
    mine = shard_shots(len(shots), rank, world)
    ups, downs = _per_shot(p, shots, mine)
    s1 = np.sum(ups, axis=0) if ups else 0
    s2 = np.sum(downs, axis=0) if downs else 0
    img, ill = combine_stacks(s1, s2, len(shots), True, group=dist.group.WORLD)
    if rank == 0:
        np.save(out, np.stack([img, ill]))
    dist.destroy_process_group()


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def test_two_rank_stack_equals_single(tmp_path):
    out = str(tmp_path / "img.npy")
    mp.start_processes(_worker, args=(2, _free_port(), out), nprocs=2, start_method="spawn")
    got = np.load(out)
    p = _problem()
    shots = _shots(p)
    ups, downs = _per_shot(p, shots, range(len(shots)))
    img, ill = combine_stacks(np.sum(ups, 0), np.sum(downs, 0), len(shots), True)
    assert np.allclose(got[0], img, rtol=1e-6, atol=0)
    assert np.allclose(got[1], ill, rtol=1e-6, atol=0)
