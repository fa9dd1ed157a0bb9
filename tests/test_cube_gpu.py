"""The cube engine on the GPU: `check --engine cuda` (every machine's full state against the
reference machine after every tick, src/check.c:52-113) on random programs with and without id and
link cells over 512 to 4096 machines, and Game of Life on the cube against plain C Life
(src/work.c:601-622) up to the full 65,536-machine, 8192 x 8192 board."""
import random

import numpy as np
import pytest

import oracle as O
import tesseract_gb300 as T
from cube_cases import random_link_program
from tesseract_gb300.life import LifeCube, pack_rows, unpack_rows

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", range(12))
def test_check_random_plain_programs(seed):
    """Random programs without links (tests/test_jit.c:173-200 style), 512 machines."""
    rnd = random.Random(seed)
    p = T.Program.random(rnd.randrange(1, 400), rnd.randrange(1, 3000), seed)
    r = T.check(p, seed=seed + 1, ticks=3)
    assert r["ok"], r
    assert r["compared"] == 512 * 4


@pytest.mark.parametrize("seed,dims", [(s, d) for s in range(6) for d in (9, 10, 11, 12)])
def test_check_random_link_programs(seed, dims):
    text = random_link_program(seed * 31 + dims, dims, cells=6 + seed * 5, links=4 + seed * 3,
                               length=40 + seed * 60)
    p = T.Program.from_asm(text)
    assert p.dims() == dims
    r = T.check(p, seed=seed + 7, ticks=4)
    assert r["ok"], (r, text)
    assert r["compared"] == (1 << dims) * 5


@pytest.fixture
def split_every_cell():
    """Kernels split over as many warps per word as they can (one written cell per warp, up to
    8), so that the block barrier and the per-warp cones are exercised on small programs."""
    import ctypes as C
    groups = C.c_int.in_dll(T.lib(), "tc_cube_groups")
    cells = C.c_int.in_dll(T.lib(), "tc_cube_min_cells")
    old = groups.value, cells.value
    groups.value, cells.value = 8, 1
    yield
    groups.value, cells.value = old


@pytest.mark.parametrize("seed,dims", [(s, d) for s in range(6) for d in (11, 12, 13)])
def test_check_random_link_programs_split(seed, dims, split_every_cell):
    text = random_link_program(seed * 57 + dims, dims, cells=10 + seed * 6, links=6 + seed * 3,
                               length=200 + seed * 150)
    p = T.Program.from_asm(text)
    r = T.check(p, seed=seed + 11, ticks=4)
    assert r["ok"], (r, text)


@pytest.mark.parametrize("dims,rbits,w,h", [(12, 6, 8, 8), (14, 7, 16, 8)])
def test_life_cube_small_split(dims, rbits, w, h, split_every_cell):
    L = LifeCube(dims, rbits, w=w, h=h)
    L.seed(9)
    start = L.board()
    L.run(7)
    assert (L.board() == life_reference(start, 7)).all()


@pytest.mark.parametrize("w,h,rb,cb", [(4, 4, 5, 5), (3, 5, 6, 6), (2, 2, 4, 5)])
def test_check_life_cube_programs(w, h, rb, cb):
    p = T.Program.gen_life_cube(w, h, rb, cb)
    r = T.check(p, seed=3, ticks=3)
    assert r["ok"], r


def life_reference(board: np.ndarray, gens: int) -> np.ndarray:
    packed = pack_rows(board)
    O.life_words(packed, gens)
    return unpack_rows(packed)


def test_life_oracle_matches_life_scalar():
    """The word-parallel plain C Life the checks use equals life_scalar (src/gen.c:686-700)."""
    rng = np.random.default_rng(5)
    b = rng.integers(0, 2, size=(64, 128), dtype=np.uint8)
    want = bytearray(b.tobytes())
    for _ in range(7):
        O.life_scalar(want, 128, 64)
    got = life_reference(b, 7)
    assert (got == np.frombuffer(bytes(want), dtype=np.uint8).reshape(64, 128)).all()


@pytest.mark.parametrize("dims,rbits,gens", [(9, 4, 30), (10, 5, 25), (12, 6, 20), (14, 7, 12)])
def test_life_cube_small(dims, rbits, gens):
    L = LifeCube(dims, rbits, w=8, h=8)
    L.seed(42)
    start = L.board()
    L.run(gens)
    assert (L.board() == life_reference(start, gens)).all()


def test_life_dims16_full_board():
    """The benchmark board: 65,536 machines, 32 x 32 tiles, 8192 x 8192, seed 42."""
    L = LifeCube(16)
    assert L.board().shape == (8192, 8192)
    L.seed(42)
    start = L.board()
    L.run(10)
    assert (L.board() == life_reference(start, 10)).all()


def test_cube_tune_keeps_state_and_results():
    """cuda_cube_tune: every variant (warps and word runs per group-major block) is timed from
    the cube's present state, the state is the same afterwards, the fastest is kept, and
    generations after tuning still equal plain C Life."""
    L = LifeCube(14, w=8, h=8)  # 512 words: up to 4 runs of 4 warps' 128 words, 2 of 8 warps'
    L.seed(7)
    start = L.board()
    t = L.cube.tune(8)
    assert [(c["warps"], c["iters"]) for c in t["candidates"]] == [(4, 1), (4, 2), (4, 4), (8, 1),
                                                                    (8, 2)]
    assert (L.board() == start).all()
    timed = [c["ms"] for c in t["candidates"] if c["ms"] is not None]
    assert t["best"]["ms"] == min(timed)
    L.run(9)
    assert (L.board() == life_reference(start, 9)).all()


def test_life_dims16_tuned_1000_generations():
    """The benchmark's configuration in full: 65,536 machines, 8192 x 8192, seed 42, the tuned
    kernels, 1,000 generations, against the oracle's word-parallel plain C Life."""
    import oracle as O
    from tesseract_gb300.life import pack_rows, unpack_rows
    L = LifeCube(16)
    L.seed(42)
    t = L.cube.tune(16)
    assert len(t["candidates"]) >= 2
    start = L.board()
    L.run(1000)
    packed = pack_rows(start)
    O.life_words(packed, 1000)
    assert (unpack_rows(packed) == L.board()).all()


@pytest.mark.parametrize("dims,w", [(11, 4), (13, 8), (16, 32)])
def test_life_closing_copies_in_two_memory_variants(dims, w):
    """The board's closing copies run only in each run's last pass; the others alternate between
    the kernels of two memory variants (A's and B's memory exchanged).  Runs of 1, 2, 3, 16, 17
    and 33 generations, one after the other on the same cube (graph replays, single passes, even
    and odd endings), against plain C Life after each."""
    L = LifeCube(dims, w=w, h=w)
    assert L.cube.closing_copies >= 1
    L.seed(dims)
    board = L.board()
    for gens in (1, 2, 3, 16, 17, 33):
        L.run(gens)
        board = life_reference(board, gens)
        assert (L.board() == board).all(), gens


def test_closing_copies_off_gives_the_same_cube():
    """With the exchange switched off (tc_cube_copy_swap = 0) every pass runs its copies: the same
    boards, from one kernel set."""
    import ctypes as C
    flag = C.c_int.in_dll(T.lib(), "tc_cube_copy_swap")
    flag.value = 0
    try:
        L = LifeCube(12, w=8, h=8)
        assert L.cube.closing_copies == 0
    finally:
        flag.value = 1
    L.seed(3)
    start = L.board()
    L.run(18)
    M = LifeCube(12, w=8, h=8)
    assert M.cube.closing_copies >= 1
    M.seed(3)
    M.run(18)
    assert (L.board() == M.board()).all()
    assert (M.board() == life_reference(start, 18)).all()


def test_check_programs_that_recompute_far_reads():
    """Random programs whose plan recomputes far reads of computed cells (fewer kernels than
    with the plain cut rule): every machine's full state against the reference machine after
    every tick."""
    from test_cube_plan import recomputing_programs
    for seed, text in recomputing_programs(4, 13) + recomputing_programs(2, 12):
        p = T.Program.from_asm(text)
        r = T.check(p, seed=seed, ticks=3)
        assert r["ok"], (seed, r)


@pytest.mark.parametrize("w,h", [(8, 8), (10, 7), (3, 3)])
def test_life_512_boards_20_generations(w, h):
    """The reference's own Life test (tests/test_work.c:378-416): gen_life's w x h torus in each
    of 512 machines, every board random, 20 passes, every board against plain C Life."""
    p = T.Program.gen_life(w, h)
    cube = T.Cube(p)
    assert cube.machines == 512
    rng = np.random.default_rng(w * 10 + h)
    boards = rng.integers(0, 2, size=(512, h, w), dtype=np.uint8)
    mem, rr = cube.read()
    for i, c in enumerate(p.board):
        bits = boards[:, i // w, i % w].astype(np.uint64).reshape(-1, 32)
        mem[c] = (bits << np.arange(32, dtype=np.uint64)).sum(axis=1).astype(np.uint32)
    cube.write(mem, rr)
    cube.run(20)
    mem, _ = cube.read()
    for k in range(512):
        want = bytearray(boards[k].tobytes())
        for _ in range(20):
            O.life_scalar(want, w, h)
        got = [(int(mem[c][k // 32]) >> (k % 32)) & 1 for c in p.board]
        assert got == list(want), k


def every_mask_program(dims: int) -> str:
    """y<m> = x of machine k ^ m for every mask m < 2^dims: a trie of links (the link for m reads
    the link for m without its top bit across that bit's dimension), then a copy of each."""
    lines = [".in x"] + [".out " + " ".join("y%d" % m for m in range(i, min(i + 32, 1 << dims)))
                         for i in range(0, 1 << dims, 32)]
    name = {0: "x"}
    for m in range(1, 1 << dims):
        top = m.bit_length() - 1
        name[m] = "l%d" % m
        lines.append(".link l%d = %s @ %d" % (m, name[m ^ (1 << top)], top))
    for m in range(1 << dims):
        lines += ["NAND ZERO", "NAND " + name[m], "NAND ONE", "STO y%d" % m]
    return "\n".join(lines) + "\n"


@pytest.mark.parametrize("dims", [9, 11])
def test_every_link_mask(dims):
    """Every lane permutation a link chain can make (tests/test_cube.c:157-172 checks the 512 of
    one group): lanes inside a word, across a warp's words (shuffles) and, at 2,048 machines,
    across warps through memory, each machine's y<m> against the reference machine."""
    p = T.Program.from_asm(every_mask_program(dims))
    assert p.dims() == dims
    r = T.check(p, seed=dims, ticks=2)
    assert r["ok"], r
