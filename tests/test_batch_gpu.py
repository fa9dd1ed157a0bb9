"""The batched engine on the GPU (cuda_batch_run): many enumerations of different programs,
lengths, cell counts and input widths in one persistent launch.  Every job's result must be the
reference's (golden cases), the oracle's (random equivalences), and the same alone as in the mix."""
import random

import pytest

import oracle as O
import tesseract_gb300 as T
from cases import case_id, load, same_result, setup

pytestmark = pytest.mark.gpu

GOLDEN = [c for c in load("enum.json") if "part" not in c]


def test_batch_matches_reference_golden():
    jobs, want = [], []
    keep = []
    for c in GOLDEN:
        mode, a, b, spec, kw = setup(c)
        keep.append((a, b, spec))
        jobs.append(dict(mode=mode, a=a, b=b, spec=spec, ticks=kw["ticks"]))
        want.append(c["result"])
    got = T.batch_run(jobs)
    bad = [(case_id(c), g, w) for c, g, w in zip(GOLDEN, got, want) if not same_result(g, w)]
    assert not bad, bad[:3]


def random_jobs(n, seed, max_width=18):
    rnd = random.Random(seed)
    out = []
    for i in range(n):
        cells, width = rnd.randint(8, 64), rnd.randint(3, max_width)
        length = int(round(16 * (4096 / 16) ** rnd.random()))
        a = T.Program.random_in(cells, width, length, seed * 100000 + i)
        b = a.rewrite(i, mutate=rnd.random() < 0.3)
        out.append(dict(mode=T.EN_EQUIV, a=a, b=b, ticks=rnd.choice([1, 1, 1, 2])))
    return out


def test_batch_random_equivalences_match_oracle():
    jobs = random_jobs(120, 3)
    got = T.batch_run(jobs)
    for j, g in zip(jobs, got):
        want = O.enum_run(j["mode"], j["a"], j["b"], ticks=j["ticks"])
        assert same_result(g, want), (g, want)


def test_batch_mixed_modes_same_alone_and_in_the_mix():
    jobs = random_jobs(40, 9, max_width=20)
    m = T.Program.gen_mul(8)
    jobs.append(dict(mode=T.EN_VERIFY, a=m, spec=T.Spec(m, "p = a * b")))
    jobs.append(dict(mode=T.EN_VERIFY, a=m, spec=T.Spec(m, "p = a * b ^ (a >> 3)")))
    h = T.Program.gen_hash(20, 8)
    jobs.append(dict(mode=T.EN_SEARCH, a=h, spec=T.Spec(h, "h = %d" % O.toyhash(77, 20, 8),
                                                        False)))
    rnd = random.Random(1)
    rnd.shuffle(jobs)
    mixed = T.batch_run(jobs)
    for j, g in zip(jobs, mixed):
        alone = T.batch_run([j])[0]
        single = T.enum_run(j["mode"], j["a"], j.get("b"), j.get("spec"), ticks=j.get("ticks", 1))
        for k in ("space", "tried", "hits", "hit", "ops"):
            assert g[k] == alone[k] == single[k], (k, g, alone, single)


def test_batch_refuses_what_it_cannot_run():
    big = T.Program.random(300, 100, 1)  # two ticks: the cell interpreter, 600 cells
    with pytest.raises(T.EngineError, match="slots"):
        T.batch_run([dict(mode=T.EN_EQUIV, a=big, b=big, ticks=2)])
    # one tick: the LUT path needs slots for live values only, so this one runs
    r = T.batch_run([dict(mode=T.EN_EQUIV, a=big, b=big.rewrite(3))])[0]
    assert r["hits"] == 0
    m = T.Program.gen_mul(4)
    assert T.batch_run([]) == []
