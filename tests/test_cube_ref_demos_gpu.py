"""The reference's own 512-machine cube demos (`alpha cube`, src/cubedemo.c:344-378; programs
from its lib/cube.inc, assembled by the reference itself: tests/golden/cube512.json.gz, written
by tests/golden/make_cube_golden.py) run on the GPU cube, every machine's result against plain
Python, with the checks of src/cubedemo.c:62-306; and its collectives across groups and Life on
one board across groups (tests/test_cube.c:1130-1215).  Each listing reassembles here to the
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

    def __init__(self, name, machines=N):
        self.p = T.Program.from_asm(DEMOS[name]["program"], name)
        assert program_digest(self.p.s) == DEMOS[name]["structure"]
        self.cube = T.Cube(self.p)
        assert self.cube.machines == machines
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


@pytest.mark.parametrize("dims", [10, 11])
def test_sort_across_groups(dims):
    """lib/cube.inc's bitonic sort, CMPX8_FAR across groups: random bytes and a descending run
    (the two kinds of tests/test_cube.c:1150-1170)."""
    n = 1 << dims
    for kind in (0, 1):
        r = Run("sort%d" % dims, n)
        v = (255 - np.arange(n) % 256) if kind else np.random.default_rng(dims).integers(0, 256, n)
        r.put_vec(cells(r.p, "v", 8), v)
        r.run()
        assert (r.get_vec(cells(r.p, "v", 8)) == np.sort(v)).all(), kind


@pytest.mark.parametrize("dims", [10, 12])
def test_rank_across_groups(dims):
    """The reference's gen_rank: p = how many machines below have x = 1, t = how many in all."""
    n = 1 << dims
    r = Run("rank%d" % dims, n)
    x = (np.random.default_rng(dims).integers(0, 3, n) == 0).astype(int)
    r.put(cells(r.p, "x"), x)
    r.run()
    bits = dims + 1
    assert (r.get_vec(cells(r.p, "p", bits)) == np.concatenate([[0], np.cumsum(x)[:-1]])).all()
    assert (r.get_vec(cells(r.p, "t", bits)) == x.sum()).all()


@pytest.mark.parametrize("w,h,rb,cb,gens", [(1, 1, 5, 5, 4), (2, 3, 2, 9, 3), (4, 4, 6, 5, 3),
                                            (3, 2, 10, 0, 3)])
def test_life_shapes_across_groups(w, h, rb, cb, gens):
    """Life on one board across groups in the reference's own shapes (tests/test_cube.c:1173-1215:
    w x h tiles, 2^rbits x 2^cbits machines, a column of machines included), against plain C
    Life."""
    import oracle as O
    from tesseract_gb300.life import LifeCube, pack_rows, unpack_rows
    L = LifeCube(rb + cb, rb, w=w, h=h)
    board = (np.random.default_rng(w * 100 + h).integers(0, 3, (h << rb, w << cb)) == 0)
    L.set_board(board.astype(np.uint8))
    L.run(gens)
    if (w << cb) % 64 == 0:
        packed = pack_rows(board.astype(np.uint8))
        O.life_words(packed, gens)
        want = unpack_rows(packed)
    else:
        want = bytearray(board.astype(np.uint8).tobytes())
        for _ in range(gens):
            O.life_scalar(want, w << cb, h << rb)
        want = np.frombuffer(bytes(want), dtype=np.uint8).reshape(h << rb, w << cb)
    assert (L.board() == want).all()
