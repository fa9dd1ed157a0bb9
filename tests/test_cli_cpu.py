"""The command line (bin/alpha-cuda) on paths that need no GPU, against the reference's own
stdout, stderr and exit code (tests/golden/cli_cpu.json, made by tests/golden/make_golden.py
--cli-cpu): --merge of shares whose --raw lines the reference wrote (complete, partial, a missing
file), tester1's --merge of the reference's histogram lines (several sizes, runs without a cycle,
programs cut off by a time limit), option errors, spec errors and the enumeration's refusals.
The usage text (exit code 2) is the tool's own and only its exit code is compared."""
import os
import subprocess

import pytest

import tesseract_gb300 as T
from cases import load

HERE = os.path.dirname(os.path.abspath(__file__))
CLI = os.path.join(os.path.dirname(HERE), "tesseract_gb300", "bin", "alpha-cuda")
CASES = load("cli_cpu.json")


def programs(tmp):
    a = T.Program.random_in(12, 10, 200, 424242)
    progs = {"mul4": T.Program.gen_mul(4).text(), "mul10": T.Program.gen_mul(10).text(),
             "hash16": T.Program.gen_hash(16, 5).text(), "ra": a.text(),
             "rc": a.rewrite(5, mutate=True).text(),
             "links": ".in x\n.out y\n.link l = x @ 3\nNAND l\nSTO y\n"}
    paths = {}
    for k, v in progs.items():
        paths[k] = os.path.join(tmp, k + ".asm")
        with open(paths[k], "w") as f:
            f.write(v)
    return paths


@pytest.mark.parametrize("case", CASES, ids=[" ".join(c["args"])[:70] for c in CASES])
def test_cli_without_gpu_matches_reference(case, tmp_path):
    paths = programs(str(tmp_path))
    for i, text in enumerate(case["raws"]):
        paths["raw%d" % i] = str(tmp_path / ("raw%d" % i))
        (tmp_path / ("raw%d" % i)).write_text(text)
    args = [a.format(**paths) for a in case["args"]]
    r = subprocess.run([CLI] + args, capture_output=True, text=True, timeout=60, cwd=tmp_path)
    tmp = str(tmp_path) + "/"
    assert r.returncode == case["rc"], r.stderr
    if case["rc"] != 2:
        assert r.stdout.replace(tmp, "") == case["stdout"]
        assert r.stderr.replace(tmp, "") == case["stderr"]
