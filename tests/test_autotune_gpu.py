"""The autotuner (cuda_enum_tune): every candidate kernel of a job (threads per block 128, 256,
512; stretches of 8, 16, 32 steps) gives the same result on the probe, the chosen one becomes the
job's kernel, and the job's results after tuning -- through cuda_enum_run and the allocation-free
entry point -- are still the oracle's."""
import ctypes as C

import pytest

import oracle as O
import tesseract_gb300 as T

pytestmark = pytest.mark.gpu
KEYS = ("space", "tried", "hits", "hit", "ops")


def static_run(e):
    f = T.lib().cuda_enum_run_static
    f.argtypes = [C.POINTER(T.EnumStruct), C.POINTER(T.EnumResult), C.c_char_p, C.c_size_t]
    f.restype = C.c_int
    r, err = T.EnumResult(), C.create_string_buffer(512)
    assert f(C.byref(e), C.byref(r), err, len(err)), err.value
    return r.as_dict()


@pytest.mark.parametrize("bits,spec", [(12, "p = a * b ^ (a & 5)"), (8, "p = a * b + 1")])
def test_tuned_kernel_gives_the_oracles_result(bits, spec):
    p = T.Program.gen_mul(bits)
    s = T.Spec(p, spec)
    t = T.enum_tune(T.EN_VERIFY, p, spec=s)
    timed = [c for c in t["candidates"] if c["ms"] is not None]
    assert timed and t["best"] in timed
    assert t["best"]["ms"] == min(c["ms"] for c in timed)
    if 2 * bits >= 13:  # 13 inputs or more: the work splits into stretches, all three tried
        assert {c["step_bits"] for c in t["candidates"]} == {3, 4, 5}
    got = T.enum_run(T.EN_VERIFY, p, spec=s)
    assert T.last_launch()["block"] == t["best"]["block"]
    want = O.enum_run(T.EN_VERIFY, p, spec=s)
    for k in KEYS:
        assert got[k] == want[k], k
    e = T.make_enum(T.EN_VERIFY, p, spec=s)
    st = static_run(e)
    for k in KEYS:
        assert st[k] == want[k], k


def test_tuning_an_equivalence_and_a_share():
    a = T.Program.random_in(20, 22, 600, 99)
    b = a.rewrite(5, mutate=True)
    t = T.enum_tune(T.EN_EQUIV, a, b, part=1, parts=3)
    assert t["best"]["ms"] is not None
    got = T.enum_run(T.EN_EQUIV, a, b, part=1, parts=3)
    want = O.enum_run(T.EN_EQUIV, a, b, part=1, parts=3)
    for k in KEYS:
        assert got[k] == want[k], k
