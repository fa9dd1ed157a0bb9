"""The command line (bin/alpha-cuda) against the reference's own stdout for the same commands
(tests/golden/cli.json, made by tests/golden/make_golden.py --cli): every line equal, except what
is the engine's own by design:
  - timings: the "inputs ... threads ... s" line, the seconds/threads fields of --raw, Life's
    cell-update rate line, tester1's T1RUN line (host, threads, seconds);
  - the engine's name in check ("the lane interpreter" there, "the cuda engine" here);
  - cube demos: each row's demo, what one pass does and check verdict; the instruction and
    segment counts are of this engine's own demo programs (the same computation in its own gate
    decomposition; the reference assembles `any` and `sort` from its macro library), and the
    timing columns and header text are the GPU's;
  - super: the proof (spec, shortest length, "every shorter program was tried", the check line)
    and the program's length, not the search's node count or which of the shortest programs it
    prints; the printed program must pass the check."""
import os
import re
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
             "rr": ".in x y z\nNAND x\nNAND y\nSTO t\nNAND z\nNAND t\nSTO x\n",
             "links10": (".in x\n.out y z\n.link l = x @ 9\n.link k = l @ 2\nNAND l\nSTO y\n"
                         "NAND k\nNAND ID3\nSTO z\nNAND ID9\nSTO x\n")}
    paths = {}
    for k, v in progs.items():
        paths[k] = os.path.join(tmp, k + ".asm")
        with open(paths[k], "w") as f:
            f.write(v)
    return paths


DEMOS = ("any", "rank", "max", "sort", "pack", "anf", "walsh", "xorconv", "ring", "polymul",
         "life")
WHAT = 5 + 1 + 44  # the demo and what one pass does; then instr, segs, check, timings


def normalise(text, kind="enum"):
    out = []
    for line in text.splitlines():
        if kind == "enum" and " inputs (" in line and "input bits)" in line:
            line = line[: line.index("input bits)")]
        elif kind == "enum" and line.startswith("EN "):
            f = line.split()
            line = " ".join(f[:5] + f[7:])  # drop seconds and threads
        elif kind == "check":
            for name in ("lane interpreter", "literal compiled code", "compiled code"):
                line = line.replace("the " + name, "the cuda engine")
        elif kind == "life" and "cell updates/s" in line:
            continue
        elif kind == "cube":
            if not line.split() or line.split()[0] not in DEMOS:
                continue
            # demo, what one pass does, check: the 512-machine table has no segs column
            m = re.match(r"(\S+)\s+(.*?)\s+\d+\s+(?:\d+\s+)?(OK|WRONG)\s", line)
            line = "%s %s | %s" % m.groups()
        elif kind == "super":
            if line.startswith("    NAND ") or line.startswith("    STO "):
                line = "<instruction>"
            elif "shortest:" in line:
                line = line[: line.index(" (")]
        elif kind == "tester1" and line.startswith("T1RUN "):
            continue
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
    kind = case.get("kind", "enum")
    assert normalise(got, kind) == normalise(case["stdout"], kind)
    if kind == "super":  # the program this engine printed meets the spec
        spec = T.super_parse(args[1])
        prog = T.SuperProg()
        code = [l.split() for l in got.splitlines() if l.startswith(("    NAND ", "    STO "))]
        prog.len = len(code)
        for i, (op, cell) in enumerate(code):
            prog.code[i].op = 1 if op == "STO" else 0
            prog.code[i].cell = ("_" + cell if cell[0] == "t" and cell[1:].isdigit()
                                 else cell).encode()
        assert T.super_check(spec, prog)[0]
