"""Programs that store into their own input cells, on the GPU: equivalence and search with ticks
1 and 2 through the kernel built from CUDA C, the kernel built from PTX (one tick) and the batch,
against the oracle (which equals the reference on these jobs: tests/test_written_inputs.py)."""
import pytest

import oracle as O
import tesseract_gb300 as T
from cases import same_result, written_input_jobs

pytestmark = pytest.mark.gpu


def jobs():
    for mode, a, b, text, ticks in written_input_jobs():
        spec = T.Spec(a, text, False) if text else None
        yield dict(mode=mode, a=a, b=b, spec=spec, ticks=ticks)


def test_written_inputs_cuda_c_and_ptx():
    for j in jobs():
        want = O.enum_run(j["mode"], j["a"], j["b"], j["spec"], ticks=j["ticks"])
        got = T.enum_run(j["mode"], j["a"], j["b"], j["spec"], ticks=j["ticks"])
        assert same_result(got, want), (got, want)
        if j["ticks"] == 1:
            old = T.set_enum_quick(True)
            try:
                got = T.enum_run(j["mode"], j["a"], j["b"], j["spec"])
                assert T.last_launch()["ptx"] == 1
            finally:
                T.set_enum_quick(old)
            assert same_result(got, want), (got, want)


def test_written_inputs_in_a_batch():
    js = list(jobs())
    for got, j in zip(T.batch_run(js), js):
        want = O.enum_run(j["mode"], j["a"], j["b"], j["spec"], ticks=j["ticks"])
        assert same_result(got, want), (got, want)
