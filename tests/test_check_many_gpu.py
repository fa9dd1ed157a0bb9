"""`check --engine cuda` at the reference's own test counts: 300 random programs (the shape of
tests/test_jit.c:173-200: random NAND/STO programs over plain cells, compiled code against the
reference machine) and 150 random link programs over 512 to 4,096 machines (the shape of
tests/test_cube.c:198-241).  Every machine's full state is compared with the reference machine
after every tick."""
import random

import pytest

import tesseract_gb300 as T
from cube_cases import random_link_program

pytestmark = pytest.mark.gpu


def test_300_random_programs():
    bad = []
    for seed in range(300):
        rnd = random.Random(1000 + seed)
        cells = rnd.randint(3, 40)
        p = T.Program.random(cells, rnd.randint(1, 300), 1000 + seed)
        r = T.check(p, seed=seed, ticks=3)
        if not r["ok"]:
            bad.append((seed, r))
    assert not bad, bad[:3]


def test_150_random_link_programs():
    bad = []
    for seed in range(150):
        rnd = random.Random(2000 + seed)
        dims = 9 + seed % 4
        text = random_link_program(2000 + seed, dims, cells=rnd.randint(4, 30),
                                   links=rnd.randint(2, 20), length=rnd.randint(20, 400))
        p = T.Program.from_asm(text)
        r = T.check(p, seed=seed, ticks=3)
        if not r["ok"]:
            bad.append((seed, dims, r))
    assert not bad, bad[:3]


def test_60_big_random_programs_with_read_only_stores():
    """The shape of tests/test_cube.c:934-1000: 1,024 to 4,096 machines, half of the links across
    groups, chains of links, stores to constants, ids and links mixed in (ignored)."""
    from cube_cases import big_random_program
    bad = []
    for k in range(60):
        p, dims = big_random_program(0xB16 + k)
        assert p.dims() == dims
        r = T.check(p, seed=900 + k, ticks=3)
        if not r["ok"]:
            bad.append((k, dims, r))
    assert not bad, bad[:3]
