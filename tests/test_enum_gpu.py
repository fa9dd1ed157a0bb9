"""verify / equiv / search on the GPU through the C ABI (cuda_enum_run), against the reference.

Small and medium cases are compared bit for bit (hit count, the 16 smallest hits, assignments
tried, ops) with the reference's golden outputs and with the oracle; the full-size workload
(gen mul --bits 16 over all 2^32 assignments) is checked through size-independent properties:
zero mismatches against the true spec, every assignment a mismatch against a spec off by one
(so the 16 smallest hits are 0..15), and a share split that adds up to the whole."""
import pytest

import oracle as O
import tesseract_gb300 as T
from cases import case_id, load, same_result, setup

pytestmark = pytest.mark.gpu
CASES = load("enum.json")


@pytest.mark.parametrize("case", CASES, ids=[case_id(c) for c in CASES])
def test_gpu_matches_reference_golden(case):
    mode, a, b, spec, kw = setup(case)
    got = T.enum_run(mode, a, b, spec, **kw)
    assert same_result(got, case["result"]), (got, case["result"])


def test_gpu_equals_oracle_on_random_equivalences():
    """Twenty random program pairs with inputs, 14..22 bits, identity-rewritten and mutated."""
    for seed in range(20):
        cells, width, length = 8 + (seed * 7) % 57, 14 + seed % 9, 16 + (seed * 331) % 3000
        a = T.Program.random_in(cells, width, length, seed)
        for mutate in (False, True):
            b = a.rewrite(seed + 100, mutate)
            got = T.enum_run(T.EN_EQUIV, a, b)
            want = O.enum_run(T.EN_EQUIV, a, b)
            assert same_result(got, want), (seed, mutate, got, want)
            if not mutate:
                assert got["hits"] == 0


@pytest.mark.parametrize("text", ["p = a * b", "p = a * b + a", "p = a * b - 3 * a + 1",
                                  "p = a * b ^ 1", "p = (a + 1) * b", "p = a * b << 3",
                                  "p = a * b * 3 - b"])
@pytest.mark.parametrize("parts", [1, 3])
def test_hoisted_kernels_equal_oracle(text, parts):
    """A 12 x 12 multiplier (24 inputs) runs in the permuted order with the stretch-invariant LUTs
    hoisted; the separable specs also take the bit-sliced difference path.  Hit counts, the 16
    smallest hits (sorted insertion per warp) and shares equal the oracle's."""
    p = T.Program.gen_mul(12)
    spec = T.Spec(p, text)
    for part in range(parts):
        got = T.enum_run(T.EN_VERIFY, p, spec=spec, part=part, parts=parts)
        want = O.enum_run(T.EN_VERIFY, p, spec=spec, part=part, parts=parts)
        assert same_result(got, want), (text, part, got, want)


@pytest.mark.parametrize("text", ["p = a * b", "p = a * b + 1"])
def test_hoisted_kernels_40_inputs_on_shares(text):
    """A 20 x 20 multiplier (40 inputs: words past 32 bits) with the stretch-invariant LUTs hoisted,
    run on a few of 2^20 shares (32 chunks each) and compared with the oracle's same shares."""
    p = T.Program.gen_mul(20)
    spec = T.Spec(p, text)
    for part in (0, 7, (1 << 20) - 1):
        got = T.enum_run(T.EN_VERIFY, p, spec=spec, part=part, parts=1 << 20)
        want = O.enum_run(T.EN_VERIFY, p, spec=spec, part=part, parts=1 << 20)
        assert same_result(got, want), (text, part, got, want)


def test_random_specs_equal_oracle():
    """Forty random specs on a 12 x 12 multiplier (24 inputs, permuted and hoisted), whole space
    and a 3-way share: the GPU's hits, 16 smallest and counts equal the oracle's."""
    import random
    from cases import random_spec
    r = random.Random(77)
    p = T.Program.gen_mul(12)
    for i in range(40):
        text = random_spec(r)
        spec = T.Spec(p, text)
        part, parts = (i % 3, 3) if i % 4 == 0 else (0, 1)
        got = T.enum_run(T.EN_VERIFY, p, spec=spec, part=part, parts=parts)
        want = O.enum_run(T.EN_VERIFY, p, spec=spec, part=part, parts=parts)
        assert same_result(got, want), (text, got, want)


@pytest.mark.parametrize("bits", [10, 12])
def test_hoisted_equiv_and_search_equal_oracle(bits):
    """Equivalence of a multiplier with its identity-rewritten and mutated copies, and searches
    for products, run with the hoisted (and permuted) layout: equal to the oracle."""
    p = T.Program.gen_mul(bits)
    for seed, mutate in ((3, False), (4, True), (5, True)):
        q = p.rewrite(seed, mutate)
        got = T.enum_run(T.EN_EQUIV, p, q)
        want = O.enum_run(T.EN_EQUIV, p, q)
        assert same_result(got, want), (bits, seed, mutate, got, want)
    for target in (0, 77 * 91, (1 << (2 * bits)) - 1 - 5):
        spec = T.Spec(p, "p = %d" % target, False)
        got = T.enum_run(T.EN_SEARCH, p, spec=spec)
        want = O.enum_run(T.EN_SEARCH, p, spec=spec)
        assert same_result(got, want), (bits, target, got, want)


def test_mul16_verify_full_space():
    p = T.Program.gen_mul(16)
    r = T.enum_run(T.EN_VERIFY, p, spec=T.Spec(p, "p = a * b"))
    assert r["space"] == 1 << 32 and r["tried"] == 1 << 32
    assert r["hits"] == 0 and r["hit"] == []
    assert r["ops"] == 6040 * (1 << 32)


def test_mul16_verify_every_input_wrong():
    p = T.Program.gen_mul(16)
    r = T.enum_run(T.EN_VERIFY, p, spec=T.Spec(p, "p = a * b + 1"))
    assert r["hits"] == 1 << 32 and r["hit"] == list(range(16))


def test_mul16_shares_add_up():
    p = T.Program.gen_mul(16)
    s = T.Spec(p, "p = a * b ^ (b & 1)")
    whole = T.enum_run(T.EN_VERIFY, p, spec=s)
    parts = [T.enum_run(T.EN_VERIFY, p, spec=s, part=i, part_end=j, parts=5)
             for i, j in ((0, 1), (2, 2), (3, 4))]
    assert sum(r["tried"] for r in parts) == 1 << 32
    assert sum(r["hits"] for r in parts) == whole["hits"] == 1 << 31
    merged = sorted(h for r in parts for h in r["hit"])[:16]
    assert merged == whole["hit"]


def test_toyhash32_search():
    """alpha search on gen hash --bits 32 --rounds 8: every preimage of toyhash(0xc0ffee42)."""
    p = T.Program.gen_hash(32, 8)
    x = 0xC0FFEE42
    target = O.toyhash(x, 32, 8)
    r = T.enum_run(T.EN_SEARCH, p, spec=T.Spec(p, "h = %d" % target, False))
    rev = int(format(x, "032b")[::-1], 2)  # x0 is input 0, the highest bit of the assignment
    assert rev in r["hit"]
    for h in r["hit"]:
        assert O.toyhash(int(format(h, "032b")[::-1], 2), 32, 8) == target


def test_refusals_on_gpu():
    p = T.Program.from_asm(".in a\n.out o\nNAND ID3\nSTO o\n")
    with pytest.raises(T.EngineError, match="id and link cells"):
        T.enum_run(T.EN_SEARCH, p, spec=T.Spec(p, "o = 1", False))
    q = T.Program.gen_mul(4)
    with pytest.raises(T.EngineError, match="bad --part"):
        T.enum_run(T.EN_VERIFY, q, spec=T.Spec(q, "p = a * b"), ticks=0)


def test_edge_widths():
    """0, 1 and 5 inputs (less than one 32-lane word), and a program of length 0."""
    for text, spec in ((".out o\nNAND ZERO\nSTO o\n", "o = 1"),
                       (".in a\n.out o\nNAND a\nSTO o\n", "o = ~a"),
                       (".in a b c d e\n.out o\nNAND a\nNAND b\nSTO o\n", "o = 0"),
                       (".in a\n.out a\n", "a = a")):
        p = T.Program.from_asm(text)
        s = T.Spec(p, spec)
        assert same_result(T.enum_run(T.EN_VERIFY, p, spec=s), O.enum_ref(T.EN_VERIFY, p, spec=s))
