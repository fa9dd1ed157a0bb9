"""Equivalence on the GPU with inputs and outputs matched by name (src/enum.c:48-78): pairs whose
second program declares them in another order, both ways round, through the kernel built from
CUDA C, the kernel built from PTX and the batch, against the oracle (which equals the reference
on these pairs: tests/test_equiv_names.py)."""
import pytest

import oracle as O
import tesseract_gb300 as T
from cases import reordered_pairs, same_result

pytestmark = pytest.mark.gpu


def both_ways():
    for a, b, _ in reordered_pairs():
        yield a, b
        yield b, a


def test_reordered_declarations_cuda_c_and_ptx():
    for x, y in both_ways():
        want = O.enum_run(T.EN_EQUIV, x, y)
        assert same_result(T.enum_run(T.EN_EQUIV, x, y), want)
        old = T.set_enum_quick(True)
        try:
            got = T.enum_run(T.EN_EQUIV, x, y)
            assert T.last_launch()["ptx"] == 1
        finally:
            T.set_enum_quick(old)
        assert same_result(got, want), (got, want)


def test_reordered_declarations_in_a_batch():
    pairs = list(both_ways())
    got = T.batch_run([dict(mode=T.EN_EQUIV, a=x, b=y) for x, y in pairs])
    for r, (x, y) in zip(got, pairs):
        want = O.enum_run(T.EN_EQUIV, x, y)
        assert same_result(r, want), (r, want)
