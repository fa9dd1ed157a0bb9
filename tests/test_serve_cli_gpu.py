"""`alpha-cuda serve JOBFILE`: a job list (arrival time, then a verify / equiv / search command
line) served by cuda_serve_run, every job's result in the reference's --raw wire format; each
must equal the same command run alone with --raw (which tests/golden/cli.json pins to the
reference)."""
import os
import subprocess

import pytest

import tesseract_gb300 as T

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
CLI = os.path.join(os.path.dirname(HERE), "tesseract_gb300", "bin", "alpha-cuda")


def raw_fields(lines):
    """EN mode space tried hits ops, then the hits (seconds and threads dropped)."""
    out = []
    for l in lines:
        f = l.split()
        if f[0] == "EN":
            out.append(" ".join(f[:5] + f[7:]))
        elif f[0] == "ENHIT":
            out.append(l)
    return out


@pytest.mark.parametrize("route", [[], ["--interpreter"], ["--compiled"]])
def test_served_jobs_equal_single_commands(tmp_path, route):
    progs = {"m8": T.Program.gen_mul(8), "m10": T.Program.gen_mul(10),
             "h16": T.Program.gen_hash(16, 5), "ra": T.Program.random_in(12, 14, 300, 9)}
    progs["rb"] = progs["ra"].rewrite(4, mutate=True)
    for k, p in progs.items():
        (tmp_path / (k + ".asm")).write_text(p.text())
    target = T.lib().tc_toyhash(4242, 16, 5)
    cmds = [
        ["verify", "m8.asm", "--spec", "p = a * b"],
        ["verify", "m10.asm", "--spec", "p = a * b ^ (a & 5)"],
        ["search", "h16.asm", "--want", "h = %d" % target],
        ["equiv", "ra.asm", "rb.asm"],
        ["equiv", "ra.asm", "ra.asm"],
        ["verify", "m8.asm", "--spec", "p = a * b + 1", "--ticks", "2"],
    ]
    lines = []
    for i, c in enumerate(cmds):
        q = ['"%s"' % a if " " in a else a for a in c]
        lines.append("%.3f %s" % (0.01 * i, " ".join(q)))
    (tmp_path / "jobs.txt").write_text("\n".join(lines) + "\n")
    r = subprocess.run([CLI, "serve", "jobs.txt"] + route, capture_output=True, text=True,
                       timeout=600, cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    per_job, cur = [], None
    for l in r.stdout.splitlines():
        if l.startswith("JOB "):
            cur = []
            per_job.append(cur)
            f = l.split()
            assert float(f[2]) <= float(f[3]) + 1e-6 <= float(f[4]) + 2e-6
        else:
            cur.append(l)
    assert len(per_job) == len(cmds)
    for c, got in zip(cmds, per_job):
        alone = subprocess.run([CLI] + c + ["--raw"], capture_output=True, text=True,
                               timeout=300, cwd=tmp_path)
        assert raw_fields(got) == raw_fields(alone.stdout.splitlines()), c
