"""The command line (bin/alpha-cuda) against the reference's own stdout for the same commands
(tests/golden/cli.json, made by tests/golden/make_golden.py --cli): every line equal, except the
timing part of the "inputs ... threads ... s" line and the seconds/threads fields of --raw."""
import os
import subprocess
import tempfile

import pytest

import tesseract_gb300 as T
from cases import load

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
CLI = os.path.join(os.path.dirname(HERE), "tesseract_gb300", "bin", "alpha-cuda")
CASES = load("cli.json")


def programs(tmp):
    a = T.Program.random_in(12, 10, 200, 424242)
    progs = {"mul4": T.Program.gen_mul(4).text(), "mul5": T.Program.gen_mul(5).text(),
             "mul6": T.Program.gen_mul(6).text(), "hash16": T.Program.gen_hash(16, 5).text(),
             "ra": a.text(), "rb": a.rewrite(5).text(), "rc": a.rewrite(5, mutate=True).text(),
             "mul3": T.Program.gen_mul(3).text(), "rt": T.Program.random_in(6, 5, 40, 7).text(),
             "rr": ".in x y z\nNAND x\nNAND y\nSTO t\nNAND z\nNAND t\nSTO x\n"}
    paths = {}
    for k, v in progs.items():
        paths[k] = os.path.join(tmp, k + ".asm")
        with open(paths[k], "w") as f:
            f.write(v)
    return paths


def normalise(text):
    out = []
    for line in text.splitlines():
        if " inputs (" in line and "input bits)" in line:
            line = line[: line.index("input bits)")]
        elif line.startswith("EN "):
            f = line.split()
            line = " ".join(f[:5] + f[7:])  # drop seconds and threads
        out.append(line)
    return out


@pytest.mark.parametrize("case", CASES, ids=[" ".join(c["args"]) for c in CASES])
def test_cli_matches_reference(case):
    with tempfile.TemporaryDirectory() as tmp:
        paths = programs(tmp)
        args = [a.format(**paths) for a in case["args"]]
        r = subprocess.run([CLI] + args, capture_output=True, text=True, timeout=300)
        got = r.stdout.replace(tmp + "/", "")
    assert r.returncode == case["rc"], r.stderr
    assert normalise(got) == normalise(case["stdout"])
