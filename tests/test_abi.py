"""The C ABI: the shared library loads without a GPU and exports every function that
include/*.h declares; the layouts the reference's structs must share are checked by size."""
import ctypes as C
import os
import re

import tesseract_gb300 as T

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*[A-Za-z_][\w \*]*?\b((?:cuda|tc)_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_every_declared_symbol_is_exported():
    lib = T.lib()
    names = declared()
    assert len(names) > 40
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_struct_sizes_match_the_reference_layouts():
    """LP64 sizes of the reference's structs, from compiling its headers (src/isa.h Instr,
    CellInfo, Program; src/enum.h Enum, EnumResult; src/check.h CheckResult; src/super.h
    SuperSpec, SuperProg, SuperResult): 8 8 72 72 184 56 936 1604 1640."""
    got = [C.sizeof(x) for x in (T.Instr, T.CellInfo, T.ProgramStruct, T.EnumStruct,
                                 T.EnumResult, T.CheckResult, T.SuperSpec, T.SuperProg,
                                 T.SuperResult)]
    assert got == [8, 8, 72, 72, 184, 56, 936, 1604, 1640]


def test_no_gpu_calls_fail_cleanly_without_a_gpu():
    """Without a device the engine reports an error instead of falling back to the CPU."""
    import pytest
    if os.path.exists("/dev/nvidia0"):
        pytest.skip("a GPU is present")
    p = T.Program.gen_mul(4)
    with pytest.raises(T.EngineError, match="CUDA"):
        T.enum_run(T.EN_VERIFY, p, spec=T.Spec(p, "p = a * b"))


def test_enum_add_hit_keeps_the_sixteen_smallest():
    """cuda_enum_add_hit against a plain model of enum_add_hit (src/enum.c:31-46): hits in any
    order, repeats included, leave the 16 smallest in ascending order."""
    import ctypes as C
    import random
    L = T.lib()
    L.cuda_enum_add_hit.argtypes = [C.POINTER(T.EnumResult), C.c_uint64]
    rng = random.Random(8)
    for trial in range(300):
        r, model = T.EnumResult(), []
        for _ in range(rng.randint(0, 60)):
            x = rng.randrange(40 if trial % 3 == 0 else 2**64)
            L.cuda_enum_add_hit(C.byref(r), x)
            model = sorted(model + [x])[:16]
        assert [r.hit[i] for i in range(r.nhit)] == model
