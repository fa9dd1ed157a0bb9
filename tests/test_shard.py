"""Sharding across ranks on the CPU: two gloo ranks each enumerate their share (the oracle's
enumerator stands in for the GPU, which this host does not have), gather the result records
and merge them with the engine's merge (cuda_enum_merge); the total must equal one whole run,
as the reference's --part shares merged by --merge equal the whole (tests/test_work.c:269-290)."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

import oracle as O
import tesseract_gb300 as T
from tesseract_gb300 import shard

KEYS = ("space", "tried", "hits", "hit", "ops")


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def jobs():
    m = T.Program.gen_mul(7)
    h = T.Program.gen_hash(16, 5)
    a = T.Program.random_in(10, 12, 200, 77)
    return [
        (T.EN_VERIFY, m, None, T.Spec(m, "p = a * b ^ (b & 3)")),
        (T.EN_SEARCH, h, None, T.Spec(h, "h = %d" % T.lib().tc_toyhash(999, 16, 5), False)),
        (T.EN_EQUIV, a, a.rewrite(3, mutate=True), None),
    ]


def rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        totals = []
        for mode, a, b, spec in jobs():
            s = shard.share(rank, world)
            local = O.enum_run(mode, a, b, spec, **s)
            totals.append(shard.gather_merge(local))
        out[rank] = totals
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_shares_over_gloo_merge_to_the_whole(world):
    port = free_port()
    with mp.get_context("spawn").Manager() as mgr:  # no fork after the GPU is in use
        out = mgr.dict()
        mp.spawn(rank_main, args=(world, port, out), nprocs=world, join=True)
        results = dict(out)
    for i, (mode, a, b, spec) in enumerate(jobs()):
        whole = O.enum_run(mode, a, b, spec)
        for r in range(world):
            got = results[r][i]
            for k in KEYS:
                assert got[k] == whole[k], (i, r, k, got[k], whole[k])


def test_share_rule():
    assert shard.share(1, 4) == dict(part=1, part_end=1, parts=4)
    with pytest.raises(ValueError):
        shard.share(4, 4)


def gpu_rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        out[rank] = [shard.gather_merge(shard.run_share(mode, a, b, spec, rank=rank, world=world))
                     for mode, a, b, spec in jobs()]
    finally:
        dist.destroy_process_group()


@pytest.mark.gpu
@pytest.mark.parametrize("world", [2, 3])
def test_gpu_shares_over_gloo_merge_to_the_whole(world):
    """The same over the real path: each gloo rank runs its share on the GPU (cuda_enum_run with
    --part rank/world; the ranks share this host's one GPU, and no rank's kernel waits on
    another's), gathers the records and merges them; every rank's total equals the oracle's
    whole run."""
    port = free_port()
    with mp.get_context("spawn").Manager() as mgr:
        out = mgr.dict()
        mp.spawn(gpu_rank_main, args=(world, port, out), nprocs=world, join=True)
        results = dict(out)
    for i, (mode, a, b, spec) in enumerate(jobs()):
        whole = O.enum_run(mode, a, b, spec)
        for r in range(world):
            for k in KEYS:
                assert results[r][i][k] == whole[k], (i, r, k)
