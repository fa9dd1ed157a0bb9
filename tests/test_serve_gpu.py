"""Serving with continuous batching (cuda_serve_run): a Poisson stream of mixed verify / equiv /
search jobs; every result must equal the same job run alone (batched engine, one job) and on the
plain engine (one generated kernel per job), and every job must have started after it arrived."""
import pytest

import tesseract_gb300 as T
from tesseract_gb300.workloads import serve_stream

pytestmark = pytest.mark.gpu

KEYS = ("space", "tried", "hits", "hit", "ops")


def test_served_results_equal_alone_and_plain():
    jobs, arrivals = serve_stream(48, rate=400.0, seed=7, max_width=20)
    res, start, finish = T.serve_run(jobs, arrivals, streams=3, max_wave_jobs=8)
    for j, r, a, s, f in zip(jobs, res, arrivals, start, finish):
        assert a <= s + 1e-6 and s <= f
        alone = T.batch_run([j])[0]
        plain = T.enum_run(j["mode"], j["a"], j.get("b"), j.get("spec"))
        for k in KEYS:
            assert r[k] == alone[k] == plain[k], (j["kind"], k, r[k], alone[k], plain[k])


def test_admission_by_footprint_and_slots():
    """A tight footprint and one job in flight at a time still serve every job correctly."""
    jobs, arrivals = serve_stream(12, rate=1000.0, seed=3, max_width=18)
    res, start, finish = T.serve_run(jobs, arrivals, streams=2, max_inflight_jobs=1,
                                     max_device_bytes=1, route=T.SERVE_INTERPRETER)
    order = sorted(range(len(jobs)), key=lambda i: start[i])
    for a, b in zip(order, order[1:]):
        assert finish[a] <= start[b] + 1e-6  # one job at a time
    for j, r in zip(jobs, res):
        alone = T.batch_run([j])[0]
        assert all(r[k] == alone[k] for k in KEYS)


def test_served_on_generated_kernels_equal_plain():
    """Every job routed to the generated-kernel engine: compile threads, slots on their own
    streams, results read from the pinned copy of each launch's workspace."""
    jobs, arrivals = serve_stream(20, rate=500.0, seed=11, max_width=24)
    engines = []
    res, start, finish = T.serve_run(jobs, arrivals, route=T.SERVE_COMPILED, compile_threads=3,
                                     compiled_slots=2, engines=engines)
    assert engines == [1] * len(jobs)
    for j, r, a, s, f in zip(jobs, res, arrivals, start, finish):
        assert a <= s + 1e-6 and s <= f
        plain = T.enum_run(j["mode"], j["a"], j.get("b"), j.get("spec"))
        for k in KEYS:
            assert r[k] == plain[k], (j["kind"], k, r[k], plain[k])


def test_automatic_routing_mixes_engines():
    """Wide jobs go to generated kernels, narrow ones to interpreter waves, in one stream."""
    jobs, arrivals = serve_stream(40, rate=400.0, seed=5, max_width=30, min_width=16)
    engines = []
    res, _, _ = T.serve_run(jobs, arrivals, engines=engines)
    assert 0 < sum(engines) < len(jobs), engines
    for j, r, e in zip(jobs, res, engines):
        alone = T.batch_run([j])[0]
        for k in KEYS:
            assert r[k] == alone[k], (j["kind"], e, k, r[k], alone[k])
