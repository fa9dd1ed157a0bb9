"""Pins the oracle: its enumeration against the reference's golden outputs (tests/golden/enum.json,
made by the reference binary), against the reference machine run one assignment at a time, and
against the reference's own known-answer tests (tests/test_work.c:244-376)."""
import pytest

import oracle as O
import tesseract_gb300 as T
from cases import case_id, load, same_result, setup

CASES = load("enum.json")


@pytest.mark.parametrize("case", CASES, ids=[case_id(c) for c in CASES])
def test_oracle_matches_reference_golden(case):
    mode, a, b, spec, kw = setup(case)
    got = O.enum_run(mode, a, b, spec, **kw)
    assert same_result(got, case["result"]), (got, case["result"])


SMALL = [c for c in CASES if c["result"]["space"] <= 1 << 12 and "part" not in c]


@pytest.mark.parametrize("case", SMALL, ids=[case_id(c) for c in SMALL])
def test_bitsliced_oracle_equals_reference_machine(case):
    mode, a, b, spec, kw = setup(case)
    assert same_result(O.enum_run(mode, a, b, spec, **kw), O.enum_ref(mode, a, b, spec, **kw))


def test_known_answers_multipliers():
    """gen_mul 1..7 bits verify with 0 wrong and 4^bits tried (tests/test_work.c:293-300)."""
    for bits in range(1, 8):
        p = T.Program.gen_mul(bits)
        r = O.enum_run(T.EN_VERIFY, p, spec=T.Spec(p, "p = a * b"))
        assert r["hits"] == 0 and r["tried"] == 1 << (2 * bits)


def test_known_answers_hash_search():
    """Every preimage of a toy hash value, against brute force (tests/test_work.c:322-376)."""
    for bits in (3, 16):
        p = T.Program.gen_hash(bits, 5)
        target = O.toyhash(12345 % (1 << bits), bits, 5)
        want = [x for x in range(1 << bits) if O.toyhash(x, bits, 5) == target]
        r = O.enum_run(T.EN_SEARCH, p, spec=T.Spec(p, "h = %d" % target, False))
        assert r["hits"] == len(want)
        rev = lambda x: int(format(x, "0%db" % bits)[::-1], 2)  # x0 is the highest bit
        assert sorted(rev(x) for x in want)[:16] == r["hit"]


def test_refusals():
    p = T.Program.from_asm(".in a\n.out o\nNAND ID3\nSTO o\n")
    with pytest.raises(T.EngineError, match="id and link cells"):
        O.enum_run(T.EN_SEARCH, p, spec=T.Spec(p, "o = 1", False))
    q = T.Program.gen_mul(4)
    with pytest.raises(T.EngineError, match="bad --part"):
        O.enum_run(T.EN_VERIFY, q, spec=T.Spec(q, "p = a * b"), part=2, parts=2)
    wide = T.Program.from_asm(".in " + " ".join("x%d" % i for i in range(47)) + "\n.out y\n")
    with pytest.raises(T.EngineError, match="too many"):
        O.enum_run(T.EN_SEARCH, wide, spec=T.Spec(wide, "y = 1", False))
