"""Enumeration at the smallest and the largest spaces, on the GPU: programs with no inputs (one
assignment, the empty input) and with one to three inputs (fewer assignments than the 32 lanes of
a word), in every mode and with ticks 1 and 2, through cuda_enum_run and through cuda_batch_run;
and 46 inputs, the most the reference enumerates (src/enum.h EN_MAX_IN), on shares of its 2^46
assignments, checked by properties that need no CPU run of the space, with 48 refused.

The no-input results are the reference's own `--raw` lines for these programs
(src/work.c:435-443; `alpha verify|search|equiv ... --raw` run on them):
    verify ZERO_IN --spec "y = 0"        EN 0 1 1 1 ... 2048, ENHIT 0
    verify ZERO_IN --spec "y = 1"        EN 0 1 1 0 ... 2048
    search ZERO_IN --want "y = 1"        EN 2 1 1 1 ... 2048, ENHIT 0
    equiv ZERO_IN ZERO_IN2               EN 1 1 1 1 ... 3584, ENHIT 0
the others are checked against the oracle."""
import pytest

import oracle as O
import tesseract_gb300 as T
from cases import same_result

pytestmark = pytest.mark.gpu

ZERO_IN = ".out y z\nNAND ZERO\nSTO y\nNAND ONE\nSTO z\n"
ZERO_IN2 = ".out y z\nNAND ZERO\nSTO y\nSTO z\n"


def reference(hits, ops):
    return {"space": 1, "tried": 1, "hits": hits, "hit": [0] * hits, "ops": ops}


def no_input_jobs():
    p, q = T.Program.from_asm(ZERO_IN), T.Program.from_asm(ZERO_IN2)
    return [
        (dict(mode=T.EN_VERIFY, a=p, spec=T.Spec(p, "y = 0")), reference(1, 2048)),
        (dict(mode=T.EN_VERIFY, a=p, spec=T.Spec(p, "y = 1")), reference(0, 2048)),
        (dict(mode=T.EN_SEARCH, a=p, spec=T.Spec(p, "y = 1", False)), reference(1, 2048)),
        (dict(mode=T.EN_EQUIV, a=p, b=q), reference(1, 3584)),
    ]


def few_input_jobs():
    jobs = []
    for width in (1, 2, 3):
        for seed in range(3):
            a = T.Program.random_in(6 + 3 * seed, width, 40 + 37 * seed, 7000 + 10 * width + seed)
            for ticks in (1, 2):
                jobs.append(dict(mode=T.EN_EQUIV, a=a, b=a.rewrite(seed, False), ticks=ticks))
                jobs.append(dict(mode=T.EN_EQUIV, a=a, b=a.rewrite(seed, True), ticks=ticks))
    m = T.Program.gen_mul(1)  # a0, b0 -> p0 p1
    for text in ("p = a * b", "p = a + b", "p = 1"):
        jobs.append(dict(mode=T.EN_VERIFY, a=m, spec=T.Spec(m, text)))
    for target in range(4):
        jobs.append(dict(mode=T.EN_SEARCH, a=m, spec=T.Spec(m, "p = %d" % target, False)))
    return jobs


def oracle(j):
    return O.enum_run(j["mode"], j["a"], j.get("b"), j.get("spec"), ticks=j.get("ticks", 1))


def test_no_inputs_equal_the_reference():
    for j, want in no_input_jobs():
        got = T.enum_run(j["mode"], j["a"], j.get("b"), j.get("spec"))
        assert same_result(got, want), (j["mode"], got, want)
        assert same_result(oracle(j), want)


def test_one_to_three_inputs_equal_the_oracle():
    for j in few_input_jobs():
        got = T.enum_run(j["mode"], j["a"], j.get("b"), j.get("spec"), ticks=j.get("ticks", 1))
        want = oracle(j)
        assert same_result(got, want), (j["mode"], len(j["a"].inputs), got, want)


def test_smallest_spaces_in_a_batch():
    """The same jobs as one batch: each result equals the job run alone."""
    jobs = [j for j, _ in no_input_jobs()] + few_input_jobs()
    wants = [oracle(j) for j in jobs]
    for got, want in zip(T.batch_run(jobs), wants):
        assert same_result(got, want), (got, want)


def test_46_inputs_on_shares():
    """A 23 x 23 multiplier: 2^46 assignments in 2^31 chunks of 32,768, split into 2^26 shares of
    32 chunks (share s holds chunks s + k 2^26, src/enum.c:232-234).  Input a0, a's lowest bit, is
    the assignment's top bit (45).  Against the true product a share has no mismatch; against
    the product + 1 every assignment is one, the smallest 16 being its first chunk's first;
    against the product ^ (a & 1) exactly the chunks from 2^30 on (bit 45 set)."""
    p = T.Program.gen_mul(23)
    assert len(p.inputs) == 46
    parts, chunk = 1 << 26, 32768
    per = 32 * chunk
    ops = 32 * 64 * 512 * len(p)  # 64 passes of 512 lanes per chunk
    true, off, top = (T.Spec(p, t) for t in ("p = a * b", "p = a * b + 1", "p = a * b ^ (a & 1)"))
    for part in (0, 12345, parts - 1):
        r = T.enum_run(T.EN_VERIFY, p, spec=true, part=part, parts=parts)
        assert (r["space"], r["tried"], r["hits"], r["hit"], r["ops"]) == (1 << 46, per, 0, [], ops)
        r = T.enum_run(T.EN_VERIFY, p, spec=off, part=part, parts=parts)
        assert r["hits"] == per and r["hit"] == [part * chunk + i for i in range(16)], r
        r = T.enum_run(T.EN_VERIFY, p, spec=top, part=part, parts=parts)
        first = part + 16 * parts  # the share's first chunk at or past 2^30
        assert r["hits"] == 16 * chunk and r["hit"] == [first * chunk + i for i in range(16)], r


def test_48_inputs_are_refused():
    p = T.Program.gen_mul(24)
    with pytest.raises(T.EngineError, match="48 inputs is too many to try them all"):
        T.enum_run(T.EN_VERIFY, p, spec=T.Spec(p, "p = a * b"), part=0, parts=1 << 30)
