"""Equivalence matches inputs and outputs by name (src/enum.c:48-78): pairs whose second program
declares them in another order, against the reference's own `alpha equiv A B --raw` (run here
where it was built from its sources; skipped elsewhere) and the oracle, both ways round."""
import os
import subprocess

import pytest

import oracle as O
import tesseract_gb300 as T
from cases import reordered_pairs, same_result

needs_ref = pytest.mark.skipif(not O.have_reference(), reason="the reference is not built here")


def raw_result(stdout):
    r = {"hit": []}
    for line in stdout.splitlines():
        f = line.split()
        if f and f[0] == "EN":
            r.update(space=int(f[2]), tried=int(f[3]), hits=int(f[4]), ops=int(f[7]))
        elif f and f[0] == "ENHIT":
            r["hit"].append(int(f[1], 16))
    return r


@needs_ref
def test_oracle_matches_reference_on_reordered_declarations(tmp_path):
    for i, (a, b, mutate) in enumerate(reordered_pairs()):
        pa, pb = tmp_path / ("a%d.asm" % i), tmp_path / ("b%d.asm" % i)
        pa.write_text(a.text())
        pb.write_text(b.text())
        for x, y, px, py in ((a, b, pa, pb), (b, a, pb, pa)):
            out = subprocess.run([O.REF_BIN, "equiv", str(px), str(py), "--raw"],
                                 capture_output=True, text=True, timeout=120)
            assert out.returncode == 0, out.stderr
            want = raw_result(out.stdout)
            got = O.enum_run(T.EN_EQUIV, x, y)
            assert same_result(got, want), (i, got, want)
            if not mutate:
                assert want["hits"] == 0
