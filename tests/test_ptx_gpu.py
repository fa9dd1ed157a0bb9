"""The kernels built from PTX that the engine writes directly (the quick-start builds of
equivalence and search jobs, csrc/ptxgen.c) on the GPU: every equivalence and search case of the
reference's golden set (shares included), random equivalences of 8 to 26 inputs rewritten and
mutated, shares of a 40-input pair (words past 32 bits, chunks picked by the share arithmetic)
and searches, each against the reference's golden output or the oracle, with the launch
reported as a PTX build.  A batch gives the same results with its compiled jobs built from PTX as
from CUDA C."""
import pytest

import oracle as O
import tesseract_gb300 as T
from cases import case_id, load, same_result, setup

pytestmark = pytest.mark.gpu
CASES = [c for c in load("enum.json") if c["mode"] != "verify" and c.get("ticks", 1) == 1]


@pytest.fixture(autouse=True)
def quick_builds():
    old = T.set_enum_quick(True)
    yield
    T.set_enum_quick(old)


def run_ptx(*args, **kw):
    got = T.enum_run(*args, **kw)
    assert T.last_launch()["ptx"] == 1
    return got


@pytest.mark.parametrize("case", CASES, ids=[case_id(c) for c in CASES])
def test_ptx_kernel_matches_reference_golden(case):
    mode, a, b, spec, kw = setup(case)
    got = run_ptx(mode, a, b, spec, **kw)
    assert same_result(got, case["result"]), (got, case["result"])


def test_ptx_kernel_equals_oracle_on_random_equivalences():
    for seed in range(24):
        cells, width, length = 8 + (seed * 5) % 57, 8 + seed % 19, 16 + (seed * 397) % 3000
        a = T.Program.random_in(cells, width, length, 910000 + seed)
        for mutate in (False, True):
            b = a.rewrite(seed + 300, mutate)
            got = run_ptx(T.EN_EQUIV, a, b)
            want = O.enum_run(T.EN_EQUIV, a, b)
            assert same_result(got, want), (seed, mutate, got, want)
            if not mutate:
                assert got["hits"] == 0


@pytest.mark.parametrize("parts", [3, 7])
def test_ptx_kernel_shares_equal_oracle(parts):
    a = T.Program.random_in(30, 20, 1200, 920001)
    b = a.rewrite(5, True)
    for part in range(parts):
        got = run_ptx(T.EN_EQUIV, a, b, part=part, parts=parts)
        want = O.enum_run(T.EN_EQUIV, a, b, part=part, parts=parts)
        assert same_result(got, want), (part, got, want)


def test_ptx_kernel_40_inputs_on_shares():
    """40 inputs: assignment bits past 36 come from the word's high half; three of 2^20 shares
    (32 chunks each, chunk = share + k * 2^20)."""
    a = T.Program.random_in(48, 40, 1500, 920002)
    b = a.rewrite(6, True)
    for part in (0, 12345, (1 << 20) - 1):
        got = run_ptx(T.EN_EQUIV, a, b, part=part, parts=1 << 20)
        want = O.enum_run(T.EN_EQUIV, a, b, part=part, parts=1 << 20)
        assert same_result(got, want), (part, got, want)


@pytest.mark.parametrize("text", ["p = 391", "p = 0", "p = 4095"])
def test_ptx_search_equals_oracle(text):
    p = T.Program.gen_mul(12)
    spec = T.Spec(p, text, False)
    got = run_ptx(T.EN_SEARCH, p, spec=spec)
    want = O.enum_run(T.EN_SEARCH, p, spec=spec)
    assert same_result(got, want), (got, want)


def test_batch_with_ptx_builds_equals_nvrtc_builds():
    """The same 384 batched pairs, their compiled jobs built by NVRTC and then from PTX (the two
    builds are cached apart, so the second batch compiles its own): equal results, and every
    identity-rewritten pair without a hit."""
    from tesseract_gb300.workloads import batch_equiv_jobs
    jobs = batch_equiv_jobs(seeds=range(930000, 930384))
    old = T.set_enum_ptx(False)
    try:
        nvrtc = T.batch_run(jobs)
        T.set_enum_ptx(True)
        ptx = T.batch_run(jobs)
        st = T.batch_stats()
    finally:
        T.set_enum_ptx(old)
    keys = ("space", "tried", "hits", "hit", "ops")
    assert all(x[k] == y[k] for x, y in zip(nvrtc, ptx) for k in keys)
    for j, r in zip(jobs, ptx):
        if not j["mutated"]:
            assert r["hits"] == 0
    assert st["jobs"] == len(jobs) and st["compiled"] > 0


def test_batch_with_every_kernel_prepared():
    """cuda_batch_prepare compiles the quick kernels of every job worth a launch; the next batch
    of the same jobs runs each of those on its cached kernel (none compiled, none taken back) and
    gives the results of the cold batch."""
    from tesseract_gb300.workloads import batch_equiv_jobs
    T.set_enum_quick(False)
    jobs = batch_equiv_jobs(seeds=range(940000, 940256))
    cold = T.batch_run(jobs)
    n = T.batch_prepare(jobs)
    warm = T.batch_run(jobs)
    st = T.batch_stats()
    keys = ("space", "tried", "hits", "hit", "ops")
    assert all(x[k] == y[k] for x, y in zip(cold, warm) for k in keys)
    assert n > 0 and st["compiled"] == n and st["taken_back"] == 0
    assert st["compile_busy"] < 0.05 * n
