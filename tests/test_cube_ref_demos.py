"""The reference's own 512-machine cube demo programs (tests/golden/cube512.json.gz, assembled by
the reference from its lib/cube.inc) on the oracle's reference machine, no GPU: each listing
reassembles here to the reference's program (the digest of its instructions, id and link cells,
inputs and outputs), and each demo gives the results its check in
src/cubedemo.c:62-306 wants.  This pins the fixture and the expected values that
tests/test_cube_ref_demos_gpu.py holds the GPU cube to."""
import numpy as np
import pytest

import oracle as O
import tesseract_gb300 as T
from cases import load_gz, program_digest

N = 512
DEMOS = load_gz("cube512.json.gz")


def cells(p, stem, n=None):
    names = [p.s.cell_names[c].decode() for c in range(p.s.ncells)]
    if n is None:
        return names.index(stem)
    return [names.index("%s%d" % (stem, i)) for i in range(n)]


def machine(name, inputs):
    """inputs: {cell: per-machine values}; one pass on the reference machine."""
    p = T.Program.from_asm(DEMOS[name]["program"], name)
    assert program_digest(p.s) == DEMOS[name]["structure"]
    cube = O.RefCube(p, N)
    for c, vals in inputs.items():
        for k in range(N):
            cube.set(k, c, int(vals[k]))
    cube.tick()
    return p, cube


def vec(cube, cs):
    return np.array([sum(cube.get(k, c) << i for i, c in enumerate(cs)) for k in range(N)])


DIMS = {"sort10": 10, "sort11": 11, "rank10": 10, "rank12": 12}


def test_every_listing_round_trips():
    for name, d in DEMOS.items():
        p = T.Program.from_asm(d["program"], name)
        assert program_digest(p.s) == d["structure"], name
        assert p.dims() == DIMS.get(name, 9), name


def test_sort_across_groups_on_the_reference_machine():
    """lib/cube.inc's bitonic sort at 1,024 machines: CMPX8_FAR across the two groups."""
    n = 1024
    p = T.Program.from_asm(DEMOS["sort10"]["program"], "sort10")
    vc = cells(p, "v", 8)
    v = np.random.default_rng(5).integers(0, 256, n)
    cube = O.RefCube(p, n)
    for k in range(n):
        for i, c in enumerate(vc):
            cube.set(k, c, int((v[k] >> i) & 1))
    cube.tick()
    got = [sum(cube.get(k, c) << i for i, c in enumerate(vc)) for k in range(n)]
    assert got == sorted(v.tolist())


def test_sort_pack_perm():
    rnd = np.random.default_rng(11)
    v = rnd.integers(0, 256, N)
    p = T.Program.from_asm(DEMOS["sort"]["program"], "sort")
    vc = cells(p, "v", 8)
    p, cube = machine("sort", {c: (v >> i) & 1 for i, c in enumerate(vc)})
    assert (vec(cube, vc) == np.sort(v)).all()

    h = (rnd.integers(0, 10, N) == 0).astype(int)
    p = T.Program.from_asm(DEMOS["pack"]["program"], "pack")
    vc, hc = cells(p, "v", 8), cells(p, "h")
    ins = {c: (v >> i) & 1 for i, c in enumerate(vc)}
    ins[hc] = h
    p, cube = machine("pack", ins)
    hits = v[h == 1]
    assert [cube.get(k, hc) for k in range(N)] == [int(k < len(hits)) for k in range(N)]
    assert (vec(cube, vc)[:len(hits)] == hits).all()

    ctl = rnd.integers(0, 2, (17, N))
    p = T.Program.from_asm(DEMOS["perm"]["program"], "perm")
    vc = cells(p, "v", 8)
    ins = {c: (v >> i) & 1 for i, c in enumerate(vc)}
    for k in range(17):
        ins[cells(p, "c%d" % k)] = ctl[k]
    p, cube = machine("perm", ins)
    want, idx = v.copy(), np.arange(N)
    for k, d in enumerate(list(range(9)) + list(range(7, -1, -1))):
        want = np.where(ctl[k] == 1, want[idx ^ (1 << d)], want)
    assert (vec(cube, vc) == want).all()
