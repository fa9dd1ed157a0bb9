"""The superoptimizer on the GPU: the shortest program for the reference's known-answer
specifications (tests/test_super.c:159-172, 321-345), the full adder's 19 with nothing of 18 or
fewer, and every program it prints passing the reference's check (any garbage, every sharing)."""
import pytest

import tesseract_gb300 as T

pytestmark = pytest.mark.gpu

SMALL = [("RR = 1", 1), ("RR = !RR", 1), ("RR = 0", 2), ("RR = x", 3), ("RR = !x", 2),
         ("RR = RR & x", 2), ("RR = RR | x", 4), ("RR = !(RR | x)", 5), ("RR = RR & !x", 4),
         ("RR = RR | !x", 2), ("x = !RR; RR = RR", 3), ("dst = src; RR = src", 4),
         ("r = r | n", 6), ("r = r & n", 6), ("m = id & n", 6), ("o{x,y} = x & y", 6),
         ("o{x,y} = x | y", 6), ("RR = RR ^ x", 7), ("RR = !(RR ^ x)", 8), ("r = r ^ n", 8),
         ("o{x,y} = x ^ y", 8), ("r{a,b} = s ? a : b", 9)]
DEEP = [("g = a & !b | a & g | !b & g", 9), ("f = f ^ (id & n)", 12),
        ("r = (id ^ s) ? n : r", 14)]


@pytest.mark.parametrize("text,best", SMALL + DEEP)
def test_known_optima(text, best):
    r = T.super_search(text, max_cost=20)
    assert r["found"] and r["cost"] == best and r["below"] == best, r
    assert not r["contradiction"]
    assert r["checked"], r["check_error"]
    assert len(r["program"]) == best


def test_full_adder_nothing_below_16_within_15():
    """tests/test_super.c:313-315: no full adder of 15 or fewer (below == 16)."""
    r = T.super_search("s{a,b} = a ^ b ^ c; c = a&b | a&c | b&c", max_cost=15)
    assert not r["found"] and r["below"] == 16


@pytest.mark.slow
def test_full_adder_is_19():
    r = T.super_search("s{a,b} = a ^ b ^ c; c = a&b | a&c | b&c", max_cost=20)
    assert r["found"] and r["cost"] == 19 and r["below"] == 19, r
    assert r["checked"], r["check_error"]
