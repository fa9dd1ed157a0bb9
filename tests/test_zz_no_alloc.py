"""cuda_enum_run_static, the enumeration whose workspace is a fixed device array (it allocates
nothing), against cuda_enum_run on the same jobs: equal results on two calls in a row, with jobs
that leave many hits in the shared array run before jobs that find none, and small grids with
hits run right after the full 2^32 grid.  Collected last; passes alone in a fresh process and
after the other tests."""
import ctypes as C

import pytest

import tesseract_gb300 as T

pytestmark = pytest.mark.gpu

KEYS = ("space", "tried", "hits", "hit", "ops", "threads")


def run_static(e):
    f = T.lib().cuda_enum_run_static
    f.argtypes = [C.POINTER(T.EnumStruct), C.POINTER(T.EnumResult), C.c_char_p, C.c_size_t]
    f.restype = C.c_int
    r, err = T.EnumResult(), C.create_string_buffer(512)
    if not f(C.byref(e), C.byref(r), err, len(err)):
        raise T.EngineError(err.value.decode())
    return r.as_dict()


def jobs():
    mul12, mul16, mul10 = T.Program.gen_mul(12), T.Program.gen_mul(16), T.Program.gen_mul(10)
    hash16 = T.Program.gen_hash(16, 5)
    a = T.Program.random_in(16, 12, 300, 31337)
    target = T.lib().tc_toyhash(12345, 16, 5)
    return [
        # many hits: every odd a
        dict(mode=T.EN_VERIFY, a=mul12, spec=T.Spec(mul12, "p = a * b ^ (a & 1)")),
        dict(mode=T.EN_VERIFY, a=mul12, spec=T.Spec(mul12, "p = a * b")),
        dict(mode=T.EN_SEARCH, a=hash16, spec=T.Spec(hash16, "h = %d" % target, False)),
        dict(mode=T.EN_EQUIV, a=a, b=a.rewrite(7, mutate=True)),
        dict(mode=T.EN_EQUIV, a=a, b=a.rewrite(7)),
        # a share of the chunks, every assignment a hit
        dict(mode=T.EN_VERIFY, a=mul10, spec=T.Spec(mul10, "p = a * b ^ 1"), part=1, parts=3),
        # the whole 2^32 space: the full grid, no hits
        dict(mode=T.EN_VERIFY, a=mul16, spec=T.Spec(mul16, "p = a * b")),
        # then a small grid with hits: its lists must not mix with the larger launch's
        dict(mode=T.EN_VERIFY, a=mul10, spec=T.Spec(mul10, "p = a * b ^ (b & 2)")),
        dict(mode=T.EN_VERIFY, a=mul16, spec=T.Spec(mul16, "p = a * b ^ (a & 1)")),
        dict(mode=T.EN_VERIFY, a=mul10, spec=T.Spec(mul10, "p = a * b ^ (b & 2)"), part=2,
             parts=5),
    ]


def test_static_workspace_matches_cuda_enum_run_twice():
    for j in jobs():
        args = (j["mode"], j["a"], j.get("b"), j.get("spec"))
        kw = dict(part=j.get("part", 0), parts=j.get("parts", 1))
        want = T.enum_run(*args, **kw)
        e = T.make_enum(*args, **kw)
        first = run_static(e)
        second = run_static(e)
        for k in KEYS:
            assert first[k] == want[k], (k, first[k], want[k])
            assert second[k] == want[k], (k, second[k], want[k])


def test_job_without_a_loaded_kernel_is_refused():
    p = T.Program.gen_mul(7)
    spec = T.Spec(p, "p = a * b ^ 0x5a5a")  # the Enum holds only its pointer: keep it alive
    e = T.make_enum(T.EN_VERIFY, p, spec=spec)
    with pytest.raises(T.EngineError, match="cuda_enum_run first"):
        run_static(e)
