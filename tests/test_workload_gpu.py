"""The batched and served workloads, job by job, against the reference's own verdicts.

tests/golden/batch_equiv.json.gz and serve_stream.json.gz hold, for every job, what the
reference's `alpha verify|equiv|search ... --raw` printed (tests/golden/make_workload_golden.py):
space, tried, hits, ops and the 16 smallest hits.  Here the same jobs run through cuda_batch_run
(the 4,096 equivalence pairs of the batched configuration in one call) and cuda_serve_run (the
two 400-job Poisson streams, inputs up to 34 and up to 22 bits, arriving at 2,000 jobs/s), and
every job's result must be the reference's."""
import pytest

import tesseract_gb300 as T
from cases import as_record, load_gz
from tesseract_gb300.workloads import batch_equiv_jobs, serve_stream

pytestmark = pytest.mark.gpu


def test_batch_of_4096_equivalences_matches_reference():
    g = load_gz("batch_equiv.json.gz")
    jobs = batch_equiv_jobs(g["jobs"], mutate_every=g["mutate_every"])
    got = [as_record(r) for r in T.batch_run(jobs)]
    bad = [(j["seed"], w, m) for j, w, m in zip(jobs, g["results"], got) if w != m]
    assert not bad, bad[:5]
    # every negative control that finds no difference is one the reference finds none in either
    silent = [j["seed"] for j, r in zip(jobs, got) if j["mutated"] and r[2] == 0]
    assert all(g["results"][s][2] == 0 for s in silent)


@pytest.mark.parametrize("max_width", [34, 22])
def test_served_stream_matches_reference(max_width):
    g = load_gz("serve_stream.json.gz")
    want = g["streams"][str(max_width)]
    jobs, arrivals = serve_stream(len(want), rate=g["rate"], seed=g["seed"], max_width=max_width)
    engines = []
    res, start, finish = T.serve_run(jobs, arrivals, engines=engines)
    got = [as_record(r) for r in res]
    bad = [(i, w, m) for i, (w, m) in enumerate(zip(want, got)) if w != m]
    assert not bad, bad[:5]
    assert all(f >= s >= 0 for s, f in zip(start, finish))
