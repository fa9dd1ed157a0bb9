"""The big-cube demo programs (tc_gen_cube_any / rank / sort, the demos of src/cubedemo.c:398-548)
run on the oracle's reference machine (a lockstep cube, one byte per cell) and checked against
plain Python: OR over all machines, prefix counts, a sorted array.  No GPU: this pins the
generators; tests/test_cubedemo_gpu.py runs the same programs on the GPU cube."""
import random

import pytest

import oracle as O
import tesseract_gb300 as T


def cells(p, stem, n):
    names = [p.s.cell_names[c].decode() for c in range(p.s.ncells)]
    return [names.index("%s%d" % (stem, i)) for i in range(n)]


def cell(p, name):
    names = [p.s.cell_names[c].decode() for c in range(p.s.ncells)]
    return names.index(name)


def run(p, dims, setup):
    n = 1 << dims
    cube = O.RefCube(p, n)
    setup(cube)
    cube.tick()
    return cube


@pytest.mark.parametrize("dims,one", [(9, 0), (9, 300), (9, 2000), (10, 1023)])
def test_any(dims, one):
    p = T.Program.gen_cube_demo("any", dims)
    x, r = cell(p, "x"), cell(p, "r")
    n = 1 << dims
    cube = run(p, dims, lambda c: [c.set(k, x, int(k == one)) for k in range(n)])
    assert all(cube.get(k, r) == int(one < n) for k in range(n))


@pytest.mark.parametrize("dims,seed", [(9, 1), (10, 2)])
def test_rank(dims, seed):
    p = T.Program.gen_cube_demo("rank", dims)
    rnd = random.Random(seed)
    n = 1 << dims
    xs = [int(rnd.random() < 0.3) for _ in range(n)]
    x, pv, tv = cell(p, "x"), cells(p, "p", dims + 1), cells(p, "t", dims + 1)
    cube = run(p, dims, lambda c: [c.set(k, x, xs[k]) for k in range(n)])
    get = lambda k, cs: sum(cube.get(k, c) << i for i, c in enumerate(cs))
    total = sum(xs)
    for k in range(n):
        assert get(k, pv) == sum(xs[:k]) and get(k, tv) == total


@pytest.mark.parametrize("dims,seed", [(9, 3), (10, 4)])
def test_sort(dims, seed):
    p = T.Program.gen_cube_demo("sort", dims)
    rnd = random.Random(seed)
    n = 1 << dims
    vs = [rnd.randrange(256) for _ in range(n)]
    v = cells(p, "v", 8)

    def setup(c):
        for k in range(n):
            for b in range(8):
                c.set(k, v[b], (vs[k] >> b) & 1)

    cube = run(p, dims, setup)
    got = [sum(cube.get(k, v[b]) << b for b in range(8)) for k in range(n)]
    assert got == sorted(vs)


def test_sizes():
    """The programs grow as the algorithms say: dims OR steps, dims add steps, and
    dims (dims + 1) / 2 compare-exchange rounds."""
    for d in (9, 12, 16):
        assert T.Program.gen_cube_demo("any", d).dims() == d
        assert T.Program.gen_cube_demo("rank", d).dims() == d
        s = T.Program.gen_cube_demo("sort", d)
        assert s.dims() == d
        assert len(s) > d * (d + 1) // 2 * 200
