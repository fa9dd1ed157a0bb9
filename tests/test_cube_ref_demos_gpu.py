"""The reference's own 512-machine cube demos (`alpha cube`, src/cubedemo.c:344-378; programs
from its lib/cube.inc, assembled by the reference itself: tests/golden/cube512.json.gz, written
by tests/golden/make_cube_golden.py) run on the GPU cube, every machine's result against plain
Python, with the checks of src/cubedemo.c:62-306.  Each listing reassembles here to the
reference's program (the digest of its structure)."""
import random

import numpy as np
import pytest

import tesseract_gb300 as T
from cases import load_gz, program_digest

pytestmark = pytest.mark.gpu

N = 512
DEMOS = load_gz("cube512.json.gz")


def cells(p, stem, n=None):
    names = [p.s.cell_names[c].decode() for c in range(p.s.ncells)]
    if n is None:
        return names.index(stem)
    return [names.index("%s%d" % (stem, i)) for i in range(n)]


class Run:
    """A cube of the demo's program: values in per machine, one pass, values out."""

    def __init__(self, name):
        self.p = T.Program.from_asm(DEMOS[name]["program"], name)
        assert program_digest(self.p.s) == DEMOS[name]["structure"]
        self.cube = T.Cube(self.p)
        assert self.cube.machines == N
        mem, rr = self.cube.read()
        self.mem = mem.reshape(self.p.s.ncells, -1)
        self.mem[:] = 0
        self.mem[1] = 0xFFFFFFFF  # ONE
        self.rr = rr * 0

    def put(self, cell, bits):
        b = np.asarray(bits, dtype=np.uint64).reshape(-1, 32)
        self.mem[cell] = (b << np.arange(32, dtype=np.uint64)).sum(axis=1).astype(np.uint32)

    def put_vec(self, cs, vals):
        for i, c in enumerate(cs):
            self.put(c, (np.asarray(vals) >> i) & 1)

    def run(self):
        self.cube.write(self.mem.reshape(-1), self.rr)
        self.cube.run(1)
        mem, _ = self.cube.read()
        self.out = mem.reshape(self.p.s.ncells, -1)

    def get(self, cell):
        w = self.out[cell].astype(np.uint64)
        return ((w[:, None] >> np.arange(32, dtype=np.uint64)) & 1).reshape(-1).astype(np.int64)

    def get_vec(self, cs):
        return sum(self.get(c) << i for i, c in enumerate(cs))


def gray(i):
    return i ^ (i >> 1)


@pytest.mark.parametrize("seed", [1, 2])
def test_any_rank_max(seed):
    rnd = np.random.default_rng(seed)
    r = Run("any")
    x = (rnd.integers(0, 100, N) == 0).astype(int)
    r.put(cells(r.p, "x"), x)
    r.run()
    assert (r.get(cells(r.p, "r")) == int(x.any())).all()
    r = Run("rank")
    x = (rnd.integers(0, 10, N) < 3).astype(int)
    r.put(cells(r.p, "x"), x)
    r.run()
    assert (r.get_vec(cells(r.p, "p", 10)) == np.concatenate([[0], np.cumsum(x)[:-1]])).all()
    assert (r.get_vec(cells(r.p, "t", 10)) == x.sum()).all()
    r = Run("max")
    v = rnd.integers(0, 256, N)
    r.put_vec(cells(r.p, "v", 8), v)
    r.run()
    assert (r.get_vec(cells(r.p, "m", 8)) == v.max()).all()


@pytest.mark.parametrize("seed", [3, 4])
def test_sort_and_pack(seed):
    rnd = np.random.default_rng(seed)
    r = Run("sort")
    v = rnd.integers(0, 256, N)
    r.put_vec(cells(r.p, "v", 8), v)
    r.run()
    assert (r.get_vec(cells(r.p, "v", 8)) == np.sort(v)).all()
    r = Run("pack")
    v = rnd.integers(0, 256, N)
    h = (rnd.integers(0, 10, N) == 0).astype(int)
    r.put_vec(cells(r.p, "v", 8), v)
    r.put(cells(r.p, "h"), h)
    r.run()
    hits = v[h == 1]
    got_h, got_v = r.get(cells(r.p, "h")), r.get_vec(cells(r.p, "v", 8))
    assert (got_h == (np.arange(N) < len(hits))).all()
    assert (got_v[:len(hits)] == hits).all()


@pytest.mark.parametrize("seed", [5, 6])
def test_perm_network(seed):
    """PERM8: 17 rounds across dimensions 0 1 .. 8 .. 1 0, machine m taking the value of
    m ^ 2^d where its round's control bit is set (a Beneš network when the controls route a
    permutation; random controls here, simulated round by round)."""
    rnd = np.random.default_rng(seed)
    r = Run("perm")
    v = rnd.integers(0, 256, N)
    ctl = rnd.integers(0, 2, (17, N))
    r.put_vec(cells(r.p, "v", 8), v)
    for k in range(17):
        r.put(cells(r.p, "c%d" % k), ctl[k])
    r.run()
    want = v.copy()
    idx = np.arange(N)
    for k, d in enumerate(list(range(9)) + list(range(7, -1, -1))):
        want = np.where(ctl[k] == 1, want[idx ^ (1 << d)], want)
    assert (r.get_vec(cells(r.p, "v", 8)) == want).all()


@pytest.mark.parametrize("seed", [7, 8])
def test_anf_and_ring(seed):
    rnd = np.random.default_rng(seed)
    r = Run("anf")
    f = rnd.integers(0, 2, N)
    r.put(cells(r.p, "f"), f)
    r.run()
    a = f.copy()
    d = 1
    while d < N:
        a = np.where(np.arange(N) & d, a ^ a[np.arange(N) ^ d], a)
        d <<= 1
    assert (r.get(cells(r.p, "f")) == a).all()
    r = Run("ring")
    x = rnd.integers(0, 2, N)
    r.put(cells(r.p, "x"), x)
    r.run()
    want = np.zeros(N, dtype=np.int64)
    for i in range(N):
        le, c, ri = gray((i - 1) % N), gray(i), gray((i + 1) % N)
        want[c] = (110 >> ((x[le] << 2) | (x[c] << 1) | x[ri])) & 1
    assert (r.get(cells(r.p, "x")) == want).all()
