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


def failing_rank_main(rank, world, port, out, how):
    """Rank 1 fails its share (how = "raises": its enumeration raises; "corrupt": it sends a
    record without its counts; "absent": it leaves before the gather).  The others must learn
    of it on the host and raise, not hang or merge a partial total."""
    import datetime
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world,
                            timeout=datetime.timedelta(seconds=10))
    mode, a, b, spec = jobs()[0]
    try:
        if rank == 1 and how == "absent":
            out[rank] = "left"
            return
        if rank == 1 and how == "raises":
            local = {"error": "RuntimeError: the share's device is gone"}
        elif rank == 1 and how == "corrupt":
            local = {"space": 1, "hit": []}
        else:
            local = O.enum_run(mode, a, b, spec, **shard.share(rank, world))
        try:
            shard.gather_merge_checked(local)
            out[rank] = "merged"
        except shard.ShardError as e:
            out[rank] = "ShardError: " + str(e)
        except RuntimeError as e:  # the collective's timeout or a closed peer
            out[rank] = "collective failed: " + type(e).__name__
    finally:
        try:
            dist.destroy_process_group()
        except Exception:
            pass


@pytest.mark.parametrize("how", ["raises", "corrupt", "absent"])
def test_a_failed_share_is_reported_on_every_rank(how):
    world, port = 3, free_port()
    with mp.get_context("spawn").Manager() as mgr:
        out = mgr.dict()
        mp.spawn(failing_rank_main, args=(world, port, out, how), nprocs=world, join=True)
        results = dict(out)
    others = [results[r] for r in (0, 2)]
    if how == "absent":
        assert results[1] == "left"
        assert all(x.startswith("collective failed") or x.startswith("ShardError") for x in others), others
    else:
        assert all(x.startswith("ShardError: rank 1") for x in others + [results[1]]), results


def test_check_records_names_the_bad_ranks():
    good = {"space": 8, "tried": 8, "hits": 0, "hit": [], "ops": 1}
    assert shard.check_records([good, good]) == [good, good]
    with pytest.raises(shard.ShardError, match="rank 1: boom"):
        shard.check_records([good, {"error": "boom"}])
    with pytest.raises(shard.ShardError, match="rank 0: a record without tried"):
        shard.check_records([{"space": 8, "hits": 0, "hit": [], "ops": 1}, good])
    with pytest.raises(shard.ShardError, match="rank 1: no share result"):
        shard.check_records([good, None])
