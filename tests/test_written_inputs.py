"""Programs that store into their own input cells (random programs with their first cells made
inputs): the oracle against the reference's own `alpha equiv|search ... --ticks T --raw` (run
here where it was built from its sources; skipped elsewhere)."""
import subprocess

import pytest

import oracle as O
import tesseract_gb300 as T
from cases import same_result, written_input_jobs
from test_equiv_names import raw_result

needs_ref = pytest.mark.skipif(not O.have_reference(), reason="the reference is not built here")


@needs_ref
def test_oracle_matches_reference_on_written_inputs(tmp_path):
    for i, (mode, a, b, text, ticks) in enumerate(written_input_jobs()):
        pa = tmp_path / ("a%d.asm" % i)
        pa.write_text(a.text())
        if mode == T.EN_EQUIV:
            pb = tmp_path / ("b%d.asm" % i)
            pb.write_text(b.text())
            args = ["equiv", str(pa), str(pb)]
            got = O.enum_run(mode, a, b, ticks=ticks)
        else:
            args = ["search", str(pa), "--want", text]
            got = O.enum_run(mode, a, spec=T.Spec(a, text, False), ticks=ticks)
        out = subprocess.run([O.REF_BIN] + args + ["--ticks", str(ticks), "--raw"],
                             capture_output=True, text=True, timeout=120)
        assert out.returncode == 0, out.stderr
        assert same_result(got, raw_result(out.stdout)), (i, got, out.stdout[:300])
