"""Sharding an ensemble across ranks (CPU, gloo, world size 2): balanced
greedy assignment by volume and the gathered result equal to one rank's."""
import os

import numpy as np
import torch.distributed as dist
import torch.multiprocessing as mp

from flue_gb300.ensemble import NOBS, run_sharded, shard_by_volume

VOLS = [16 * 16 * 16 * 32, 24 ** 3 * 48, 32 ** 3 * 64, 16 ** 3 * 48, 24 ** 3 * 32, 32 ** 3 * 32, 24 ** 3 * 48]


def fake_compute(ids_fields):
    # stands in for the GPU ensemble: a deterministic function of the field
    return np.array([[f * 1.0, f * 2.0, f + 0.5, -f, 1.0 / (1 + f), VOLS[f]] for f in ids_fields])


def test_shard_by_volume_balances():
    shards = shard_by_volume(VOLS, 2)
    assert sorted(sum(shards, [])) == list(range(len(VOLS)))
    loads = [sum(VOLS[i] for i in s) for s in shards]
    assert max(loads) - min(loads) <= max(VOLS)
    assert shard_by_volume(VOLS, 1) == [list(range(len(VOLS)))]


def _worker(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        out = run_sharded(lambda i: i, VOLS, rank, world, compute=fake_compute)
        q.put((rank, out.tolist()))
    finally:
        dist.destroy_process_group()


def test_run_sharded_gloo_two_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    ref = fake_compute(list(range(len(VOLS))))
    for r in (0, 1):
        assert np.array_equal(np.array(res[r]), ref)
    assert ref.shape[1] == NOBS
