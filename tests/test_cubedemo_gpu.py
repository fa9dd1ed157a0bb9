"""The big-cube demos on the GPU (`alpha cube --dims D`, src/cubedemo.c:398-623): the engine's
own checked runs (every machine against plain C), the same programs through the Cube API
against Python, and `check` (every machine's full state against the reference machine after
every tick) on the demo programs themselves."""
import random

import numpy as np
import pytest

import tesseract_gb300 as T

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["any", "rank", "max", "sort", "pack", "anf", "walsh", "xorconv",
                                  "ring", "life"])
@pytest.mark.parametrize("dims", [9, 11, 16])
def test_demo_checks(name, dims):
    r = T.cube_demo(name, dims, checks=3, seconds=0.05)
    assert r["ok"], r
    assert r["passes_per_second"] > 0


@pytest.mark.parametrize("dims", [9, 11])
def test_polymul_demo(dims):
    """The NTT product mod x^N + 1 over Z_12289 against the schoolbook product."""
    r = T.cube_demo("polymul", dims, checks=2, seconds=0.05)
    assert r["ok"], r


@pytest.mark.parametrize("dims", [12, 14])
def test_sort_through_the_cube_api(dims):
    p = T.Program.gen_cube_demo("sort", dims)
    cube = T.Cube(p)
    n = cube.machines
    vals = np.random.default_rng(dims).integers(0, 256, n)
    names = [p.s.cell_names[c].decode() for c in range(p.s.ncells)]
    v = [names.index("v%d" % b) for b in range(8)]
    mem, rr = cube.read()
    mem[:] = 0
    mem[1] = 0xFFFFFFFF  # ONE
    for b in range(8):
        bits = ((vals >> b) & 1).astype(np.uint64).reshape(-1, 32)
        mem[v[b]] = (bits << np.arange(32, dtype=np.uint64)).sum(axis=1).astype(np.uint32)
    cube.write(mem, rr * 0)
    cube.run(1)
    mem, _ = cube.read()
    got = np.zeros(n, dtype=np.int64)
    for b in range(8):
        w = mem[v[b]].astype(np.uint64)
        bits = (w[:, None] >> np.arange(32, dtype=np.uint64)) & 1
        got |= bits.reshape(-1).astype(np.int64) << b
    assert (got == np.sort(vals)).all()


@pytest.mark.parametrize("name,dims", [("any", 10), ("rank", 9), ("rank", 11), ("sort", 9),
                                       ("sort", 10), ("max", 11), ("anf", 12), ("walsh", 10),
                                       ("ring", 11), ("pack", 10), ("xorconv", 9)])
def test_check_demo_programs(name, dims):
    p = T.Program.gen_cube_demo(name, dims)
    r = T.check(p, seed=dims, ticks=2)
    assert r["ok"], r
