"""Writes the reference's verdicts for the batched and served workloads, job by job.

    python tests/golden/make_workload_golden.py [batch] [serve]

Needs the reference's `alpha` built from its sources (oracle/_ref/alpha; oracle/Makefile builds
it on an x86 host that has the sources).  Each job's programs are written as assembly and run
through the reference's own command line with --raw (src/work.c:435-443), one job at a time on
all host threads:

    batch_equiv.json.gz   the 4,096 equivalence pairs of workloads.batch_equiv_jobs (seeds
                          0..4095: random programs with 16..28 inputs against copies rewritten by
                          local NAND identities, every 8th a mutated negative control)
    serve_stream.json.gz  the 400 jobs of each serving stream of workloads.serve_stream (Poisson,
                          2,000 jobs/s, seed 1; inputs up to 34 and up to 22 bits): gen mul
                          verifies, equivalences and searches for a random target

Every job is run by the reference itself; none needed the oracle.  Per job the fixture holds
[space, tried, hits, ops, "hit,hit,..."] with the 16 smallest hits in hexadecimal.
"""
from __future__ import annotations

import gzip
import json
import os
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import tesseract_gb300 as T  # noqa: E402
from tesseract_gb300.workloads import batch_equiv_jobs, serve_stream  # noqa: E402

ALPHA = os.path.join(ROOT, "oracle", "_ref", "alpha")
SERVE_STREAMS = ((34, 400), (22, 400))


def raw(args):
    r = subprocess.run([ALPHA] + args + ["--raw"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(" ".join(args) + ": " + r.stderr)
    rec, hits = None, []
    for line in r.stdout.splitlines():
        f = line.split()
        if f and f[0] == "EN":
            rec = [int(f[2]), int(f[3]), int(f[4]), int(f[7])]
        elif f and f[0] == "ENHIT":
            hits.append(f[1])
    return rec + [",".join(hits)]


def write(tmp, name, prog):
    path = os.path.join(tmp, name + ".asm")
    with open(path, "w") as f:
        f.write(prog.text())
    return path


def job_args(tmp, i, job):
    a = write(tmp, "a%d" % i, job["a"])
    if job["mode"] == T.EN_EQUIV:
        return ["equiv", a, write(tmp, "b%d" % i, job["b"])]
    verb, flag = ("verify", "--spec") if job["mode"] == T.EN_VERIFY else ("search", "--want")
    return [verb, a, flag, job["spec"].text]


def dump(name, payload):
    with gzip.open(os.path.join(HERE, name), "wt") as f:
        json.dump(payload, f, separators=(",", ":"))


def main():
    todo = [a for a in sys.argv[1:] if a in ("batch", "serve")] or ["batch", "serve"]
    with tempfile.TemporaryDirectory() as tmp:
        if "batch" in todo:
            t0 = time.time()
            jobs = batch_equiv_jobs(4096)
            res = [raw(job_args(tmp, i, j)) for i, j in enumerate(jobs)]
            dump("batch_equiv.json.gz", {"jobs": len(jobs), "mutate_every": 8, "results": res})
            print("batch: %d jobs in %.0f s" % (len(res), time.time() - t0), flush=True)
        if "serve" in todo:
            streams = {}
            for wmax, n in SERVE_STREAMS:
                t0 = time.time()
                jobs, _ = serve_stream(n, rate=2000.0, seed=1, max_width=wmax)
                streams[str(wmax)] = [raw(job_args(tmp, i, j)) for i, j in enumerate(jobs)]
                print("serve <= %d bits: %d jobs in %.0f s" % (wmax, n, time.time() - t0),
                      flush=True)
            dump("serve_stream.json.gz", {"rate": 2000.0, "seed": 1, "streams": streams})


if __name__ == "__main__":
    main()
