"""`run --table --engine cuda` (cuda_table, the replacement of table_lanes, src/main.c:297-322):
every row of random programs with inputs, 1 to 3 ticks, against the reference machine run row
by row (the oracle's lockstep cube with one machine per row), and the refusals of cmd_run."""
import random

import pytest

import oracle as O
import tesseract_gb300 as T

pytestmark = pytest.mark.gpu


def reference_table(p, ticks):
    n = p.s.ninputs
    rows = 1 << n
    cube = O.RefCube(p, rows)
    for r in range(rows):
        for k in range(n):
            cube.set(r, p.s.inputs[k], (r >> (n - 1 - k)) & 1)
    for _ in range(ticks):
        cube.tick()
    if p.s.noutputs:
        return [[cube.get(r, p.s.outputs[i]) for i in range(p.s.noutputs)] for r in range(rows)]
    return [[cube.rr(r)] for r in range(rows)]


@pytest.mark.parametrize("seed", range(10))
def test_random_programs(seed):
    rnd = random.Random(seed)
    p = T.Program.random_in(rnd.randrange(2, 24), rnd.randrange(1, 11), rnd.randrange(1, 600),
                            seed)
    ticks = 1 + seed % 3
    assert T.table(p, ticks) == reference_table(p, ticks)


def test_rr_column_and_wide_inputs():
    p = T.Program.from_asm(".in x y z\nNAND x\nNAND y\nSTO t\nNAND z\nNAND t\nSTO x\n")
    for ticks in (1, 2, 5):
        assert T.table(p, ticks) == reference_table(p, ticks)
    m = T.Program.gen_mul(6)  # inputs a0..a5 b0..b5 (a0 the row's high bit), outputs p0..p11
    got = T.table(m)
    assert len(got) == 4096
    for r in (0, 1, 77, 2048, 4095):
        bit = [(r >> (11 - k)) & 1 for k in range(12)]
        a = sum(bit[i] << i for i in range(6))
        b = sum(bit[6 + i] << i for i in range(6))
        assert sum(v << i for i, v in enumerate(got[r])) == a * b


def test_refusals():
    none = T.Program.random(6, 40, 3)  # no .in cells
    with pytest.raises(T.EngineError, match="between 1 and 20"):
        T.table(none)
    cube = T.Program.gen_life_cube(2, 2, 4, 5)
    with pytest.raises(T.EngineError, match="run as a cube"):
        T.table(cube)
