"""Enumeration across ranks: the assignment space split by the reference's share rule (chunks of
64 passes of 512 assignments, chunk c in share c mod parts, src/enum.c:11,215-242), one share per
rank, and the shares' results merged on the host as merge_raw merges --raw lines
(src/work.c:341-371, here cuda_enum_merge).  Nothing crosses ranks on the data path: each rank
enumerates its own chunks; the only exchange is the small result record, gathered once.
"""
from __future__ import annotations

import ctypes as C

import tesseract_gb300 as T


def share(rank: int, world: int) -> dict:
    """The --part arguments of rank's share: part rank of world."""
    if not 0 <= rank < world:
        raise ValueError("rank %d of %d" % (rank, world))
    return dict(part=rank, part_end=rank, parts=world)


def _struct(d: dict) -> T.EnumResult:
    r = T.EnumResult()
    r.space, r.tried, r.hits, r.ops = d["space"], d["tried"], d["hits"], d["ops"]
    r.seconds, r.threads = d.get("seconds", 0.0), d.get("threads", 0)
    r.nhit = len(d["hit"])
    for i, x in enumerate(d["hit"]):
        r.hit[i] = x
    return r


def merge(results) -> dict:
    """The total of several shares' result dicts (cuda_enum_merge)."""
    L = T.lib()
    L.cuda_enum_merge.restype = None
    L.cuda_enum_merge.argtypes = [C.POINTER(T.EnumResult), C.POINTER(T.EnumResult)]
    total = T.EnumResult()
    for d in results:
        part = _struct(d)
        L.cuda_enum_merge(C.byref(total), C.byref(part))
    return total.as_dict()


def gather_merge(local: dict, group=None) -> dict:
    """Every rank's share result, gathered over torch.distributed and merged (all ranks get
    the total)."""
    import torch.distributed as dist
    parts = [None] * dist.get_world_size(group)
    dist.all_gather_object(parts, local, group=group)
    return merge(parts)


def run_share(mode, a, b=None, spec=None, ticks=1, rank=0, world=1) -> dict:
    """This rank's share on its GPU (cuda_enum_run with --part rank/world)."""
    return T.enum_run(mode, a, b, spec, ticks, **share(rank, world))


class ShardError(RuntimeError):
    """A share failed on some rank, or a rank's record never came."""


def check_records(records) -> list:
    """The shares' records, or ShardError naming the ranks whose share failed or whose record is
    not a share result (a corrupted or missing record)."""
    bad = []
    for r, rec in enumerate(records):
        if not isinstance(rec, dict) or "error" in rec:
            bad.append("rank %d: %s" % (r, rec.get("error") if isinstance(rec, dict) else
                                        "no share result"))
        elif not all(k in rec for k in ("space", "tried", "hits", "hit", "ops")):
            bad.append("rank %d: a record without %s" % (
                r, ", ".join(k for k in ("space", "tried", "hits", "hit", "ops") if k not in rec)))
    if bad:
        raise ShardError("; ".join(bad))
    return records


def gather_merge_checked(local, group=None) -> dict:
    """gather_merge with failures reported: a rank whose share raised contributes its error
    instead of a result, and every rank raises ShardError rather than merging a partial total.
    A rank that never reaches the gather (it died, or hangs) ends the collective with the process
    group's timeout, which raises on the others."""
    import torch.distributed as dist
    parts = [None] * dist.get_world_size(group)
    dist.all_gather_object(parts, local, group=group)
    return merge(check_records(parts))


def run_share_checked(mode, a, b=None, spec=None, ticks=1, rank=0, world=1, group=None) -> dict:
    """This rank's share, gathered and merged with every rank's; a failure on any rank raises
    ShardError on all of them."""
    try:
        local = run_share(mode, a, b, spec, ticks, rank, world)
    except Exception as e:  # the share's failure goes to every rank
        local = {"error": "%s: %s" % (type(e).__name__, e)}
    return gather_merge_checked(local, group)
