"""Tester 1 on the GPU (cuda_t1_run, the replacement of t1_run, src/tester.c:235-275) against the
reference's own `tester1 --raw --threads 1` lines (tests/golden/tester1.json, made by
tests/golden/make_golden.py --tester1): programs, runs, passes, the cycle-length histogram and
the longest cycle with its program's seed, field for field."""
import os
import subprocess

import pytest

from cases import load

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
CLI = os.path.join(os.path.dirname(HERE), "tesseract_gb300", "bin", "alpha-cuda")
CASES = load("tester1.json")


def t1_lines(args):
    r = subprocess.run([CLI, "tester1"] + args + ["--raw"], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr
    assert r.stdout.startswith("T1RUN ")
    return [l for l in r.stdout.splitlines() if l.startswith("T1 ")]


@pytest.mark.parametrize("case", CASES, ids=[" ".join(c["args"]) for c in CASES])
def test_tester1_matches_reference(case):
    assert t1_lines(case["args"]) == case["t1"]


def test_merge_adds_runs(tmp_path):
    a = tmp_path / "a.txt"
    b = tmp_path / "b.txt"
    for path, seed in ((a, "1"), (b, "2")):
        r = subprocess.run([CLI, "tester1", "--cells", "8,16", "--programs", "4", "--seed", seed,
                            "--raw"], capture_output=True, text=True, timeout=300)
        path.write_text(r.stdout)
    r = subprocess.run([CLI, "tester1", "--merge", str(a), str(b)], capture_output=True,
                       text=True, timeout=60)
    assert r.returncode == 0
    assert "tester 1: 16 random programs, 8192 runs" in r.stdout
