"""The generated enumeration kernels compile for sm_103a (nvcc, no GPU needed): the device side
of the hoisted, permuted and difference-path variants, with the register report checked for
spills on the headline kernel.  Skipped where nvcc is absent."""
import os
import re
import shutil
import subprocess
import tempfile

import pytest

import tesseract_gb300 as T

NVCC = shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc"
                                if os.path.exists("/usr/local/cuda/bin/nvcc") else None)
pytestmark = pytest.mark.skipif(NVCC is None, reason="nvcc not installed")


def compile_source(src: str) -> str:
    d = tempfile.mkdtemp()
    path = os.path.join(d, "gen.cu")
    with open(path, "w") as f:
        f.write(src)
    r = subprocess.run([NVCC, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
                        "-Xptxas", "-v", "-Xptxas", "-O2", "-c", path, "-o",
                        os.path.join(d, "gen.o")], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return r.stderr


def cases():
    mul16 = T.Program.gen_mul(16)
    mul12 = T.Program.gen_mul(12)
    mul10 = T.Program.gen_mul(10)
    rnd = T.Program.random_in(24, 20, 400, 5)
    return [
        ("verify mul16 a*b", (T.EN_VERIFY, mul16, None, T.Spec(mul16, "p = a * b"), 1)),
        ("verify mul12 xor", (T.EN_VERIFY, mul12, None, T.Spec(mul12, "p = a * b ^ 1"), 1)),
        ("verify mul12 wide", (T.EN_VERIFY, mul12, None,
                               T.Spec(mul12, "p = (a * b) >> 0 | ((a * b) >> 20 << 20)"), 1)),
        ("equiv mul12", (T.EN_EQUIV, mul12, mul12.rewrite(4, True), None, 1)),
        ("search mul10", (T.EN_SEARCH, mul10, None, T.Spec(mul10, "p = 561", False), 1)),
        ("equiv random", (T.EN_EQUIV, rnd, rnd.rewrite(2), None, 1)),
        ("verify ticks 3", (T.EN_VERIFY, T.Program.gen_mul(5), None,
                            T.Spec(T.Program.gen_mul(5), "p = a * b"), 3)),
    ]


@pytest.mark.parametrize("name,args", cases(), ids=[c[0] for c in cases()])
def test_generated_kernel_compiles(name, args):
    mode, a, b, spec, ticks = args
    log = compile_source(T.codegen_enum_source(mode, a, b, spec, ticks))
    if name == "verify mul16 a*b":
        assert "0 bytes spill stores" in log and "0 bytes spill loads" in log, log
        regs = int(re.search(r"Used (\d+) registers", log).group(1))
        assert regs <= 128, log  # two blocks of 256 threads per SM


def test_grouped_kernels_compile():
    """Jobs that a compile thread builds together: one source, each job in a namespace of its own
    with its kernel renamed tc_enum_<k> and its macros undefined after it; every kernel compiles
    (ptxas -v names each entry) and the group holds the jobs' different shapes (hoisted,
    permuted, spec and equiv kernels, block sizes)."""
    import ctypes as C
    from tesseract_gb300.workloads import batch_equiv_jobs
    mul10 = T.Program.gen_mul(10)
    specs = [T.Spec(mul10, "p = a * b"), T.Spec(mul10, "p = 561", False)]
    pairs = batch_equiv_jobs(2)  # the structs point into these objects: keep them alive
    jobs = [T.make_enum(T.EN_VERIFY, mul10, None, specs[0], 1),
            T.make_enum(T.EN_SEARCH, mul10, None, specs[1], 1)]
    for j in pairs:
        jobs.append(T.make_enum(T.EN_EQUIV, j["a"], j["b"], None, 1))
    L = T.lib()
    L.tc_codegen_enum_group.restype = C.c_void_p
    L.tc_codegen_enum_group.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_size_t), C.c_char_p,
                                        C.c_size_t]
    arr = (C.POINTER(T.EnumStruct) * len(jobs))(*[C.pointer(e) for e in jobs])
    n, err = C.c_size_t(), C.create_string_buffer(256)
    ptr = L.tc_codegen_enum_group(C.cast(arr, C.c_void_p), len(jobs), C.byref(n), err, len(err))
    assert ptr, err.value
    src = C.string_at(ptr, n.value).decode()
    C.CDLL(None).free(C.c_void_p(ptr))
    assert src.count("namespace tcj") == len(jobs)
    log = compile_source(src)
    entries = set(re.findall(r"Compiling entry function '(tc_enum_\d+)'", log))
    assert entries == {"tc_enum_%d" % k for k in range(len(jobs))}, log[-2000:]
