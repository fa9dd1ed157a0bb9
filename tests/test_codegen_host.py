"""The code generator, checked on the CPU.

The engine's generated CUDA C contains a per-word function tc_word(word) -> hit mask in plain C;
these tests compile that same text with gcc (tests/host_emulation.h supplies the three CUDA
intrinsics it uses), evaluate every word of the assignment space, and compare the hit count and
the 16 smallest hits with the reference's golden results.  This checks the lowering (cells,
inputs, the specification's per-lane evaluation, the bit transpose, the comparisons) before any
GPU time is spent; the GPU tests then check the same kernels on the device."""
import ctypes as C
import os
import subprocess
import tempfile

import pytest

import tesseract_gb300 as T
from cases import case_id, load, setup

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = [c for c in load("enum.json") if c["result"]["space"] <= 1 << 22 and "part" not in c]

WRAPPER = """
void tc_host_words(unsigned long long first, unsigned long long n, unsigned *out)
{
    for (unsigned long long i = 0; i < n; i++)
        out[i] = tc_word(first + i);
}

/* every word of the space: the hit count and the 16 smallest hits, each hit's enumeration index
   y = 32 word + lane mapped back to its assignment by tc_unperm */
void tc_host_enum(unsigned long long words, unsigned long long space, unsigned long long *count,
                  unsigned long long *first, int *nfirst)
{
    unsigned long long c = 0;
    int nf = 0;
    for (unsigned long long w = 0; w < words; w++) {
        unsigned m = tc_word(w);
        if (space < 32)
            m &= (1u << space) - 1u;
        while (m) {
            const int l = __builtin_ctz(m);
            m &= m - 1u;
            c++;
            const unsigned long long x = tc_unperm((w << 5) | (unsigned long long)l);
            if (nf < 16 || x < first[15]) {
                int i = nf < 16 ? nf++ : 15;
                while (i > 0 && first[i - 1] > x) {
                    first[i] = first[i - 1];
                    i--;
                }
                first[i] = x;
            }
        }
    }
    *count = c;
    *nfirst = nf;
}
"""


def host_words(src: str):
    d = tempfile.mkdtemp()
    path = os.path.join(d, "gen.c")
    with open(path, "w") as f:
        f.write('#include "%s"\n' % os.path.join(HERE, "host_emulation.h"))
        f.write(src)
        f.write(WRAPPER)
    so = os.path.join(d, "gen.so")
    subprocess.run(["gcc", "-O1", "-std=gnu11", "-w", "-shared", "-fPIC", path, "-o", so],
                   check=True)
    L = C.CDLL(so)
    L.tc_host_words.argtypes = [C.c_uint64, C.c_uint64, C.c_void_p]
    return L


def emulate(mode, a, b, spec, kw):
    src = T.codegen_enum_source(mode, a, b, spec, kw["ticks"])
    L = host_words(src)
    L.tc_host_enum.argtypes = [C.c_uint64, C.c_uint64, C.c_void_p, C.c_void_p, C.c_void_p]
    space = 1 << len(a.inputs)
    words = (space + 31) // 32
    count, nf = C.c_uint64(), C.c_int()
    first = (C.c_uint64 * 16)()
    L.tc_host_enum(words, space, C.byref(count), first, C.byref(nf))
    return count.value, [int(first[i]) for i in range(nf.value)]


@pytest.mark.parametrize("case", CASES, ids=[case_id(c) for c in CASES])
def test_generated_code_on_host(case):
    mode, a, b, spec, kw = setup(case)
    hits, first = emulate(mode, a, b, spec, kw)
    assert hits == case["result"]["hits"]
    assert first == case["result"]["hit"]


def test_transpose_and_wide_spec_on_host():
    """A 12 x 12 multiplier checked against a 64-bit spec (two transposes, 64-bit RPN)."""
    p = T.Program.gen_mul(12)
    spec = T.Spec(p, "p = (a * b) >> 0 | ((a * b) >> 24 << 24)")
    hits, first = emulate(T.EN_VERIFY, p, None, spec, {"ticks": 1})
    assert hits == 0 and first == []


@pytest.mark.parametrize("text", ["p = a * b", "p = a * b + a", "p = a * b - 3 * a + 1",
                                  "p = a * b ^ 1", "p = a * b << 3", "p = a * b * 3 - b"])
def test_hoisted_chunk_and_spec_on_host(text):
    """A 12 x 12 multiplier (24 inputs) takes the permuted layout: b's last rows change per step,
    the rest of the LUTs run once per stretch; specs that are a sum of a step part and a lane part
    are bit-sliced once per stretch and advanced by one difference per step.  The hits and the 16
    smallest equal the oracle's."""
    import oracle as O
    p = T.Program.gen_mul(12)
    spec = T.Spec(p, text)
    src = T.codegen_enum_source(T.EN_VERIFY, p, None, spec, 1)
    assert "#define TC_PERMUTED 1" in src
    assert ("const u32 d = e[0] - sf0;" in src) == (text != "p = a * b ^ 1")
    hits, first = emulate(T.EN_VERIFY, p, None, spec, {"ticks": 1})
    want = O.enum_run(T.EN_VERIFY, p, spec=spec)
    assert hits == want["hits"] and first == want["hit"]


def test_random_specs_on_host():
    """Random specs on a 10 x 10 multiplier (20 inputs, permuted and hoisted): the separable ones
    take the difference path, the rest the per-lane path; hits and the 16 smallest equal the
    oracle's."""
    import random
    import oracle as O
    from cases import random_spec
    r = random.Random(2024)
    p = T.Program.gen_mul(10)
    for _ in range(10):
        text = random_spec(r)
        spec = T.Spec(p, text)
        hits, first = emulate(T.EN_VERIFY, p, None, spec, {"ticks": 1})
        want = O.enum_run(T.EN_VERIFY, p, spec=spec)
        assert hits == want["hits"] and first == want["hit"], text


def test_hoisted_equiv_and_search_on_host():
    """Equivalence with rewritten and mutated copies and searches for products on a 10 x 10
    multiplier, in the hoisted (permuted) layout: equal to the oracle."""
    import oracle as O
    p = T.Program.gen_mul(10)
    for seed, mutate in ((3, False), (4, True)):
        q = p.rewrite(seed, mutate)
        src = T.codegen_enum_source(T.EN_EQUIV, p, q, None, 1)
        assert "#define TC_PERMUTED 1" in src
        got = emulate(T.EN_EQUIV, p, q, None, {"ticks": 1})
        want = O.enum_run(T.EN_EQUIV, p, q)
        assert got == (want["hits"], want["hit"]), (seed, mutate)
    for target in (0, 33 * 17, (1 << 20) - 6):
        spec = T.Spec(p, "p = %d" % target, False)
        got = emulate(T.EN_SEARCH, p, None, spec, {"ticks": 1})
        want = O.enum_run(T.EN_SEARCH, p, spec=spec)
        assert got == (want["hits"], want["hit"]), target


def test_layout_choice_for_multipliers():
    """The generated enumeration code for gen mul 16: 720 LUTs, 532 of them once per stretch of
    2^4 steps in a permuted order, the spec on the difference path with 12 carry-free low bits;
    gen mul 20 (40-bit product) hoists its LUTs but keeps the per-lane spec."""
    import re
    p = T.Program.gen_mul(16)
    src = T.codegen_enum_source(T.EN_VERIFY, p, None, T.Spec(p, "p = a * b"), 1)
    assert re.search(r"// 720 LOP3 for 6040 \+ 0 NAND/STO instructions, 532 of them", src)
    assert "#define TC_STEP_BITS 4" in src and "#define TC_PERMUTED 1" in src
    assert "const u32 d = e[0] - sf0;" in src
    assert len(re.findall(r"m \|= n\d+ \^ sp\d+;", src)) == 12
    p = T.Program.gen_mul(20)
    src = T.codegen_enum_source(T.EN_VERIFY, p, None, T.Spec(p, "p = a * b"), 1)
    assert "#define TC_PERMUTED 1" in src and "sf0" not in src
    assert int(re.search(r"NAND/STO instructions, (\d+) of them", src).group(1)) > 800


def test_unperm_is_a_bijection_that_keeps_chunks():
    """tc_unperm maps the kernel's enumeration index y to the assignment x: a bijection of the
    space that moves no bit from 15 up, so every chunk of 32,768 assignments (the reference's
    --part unit) is the same set either way."""
    p = T.Program.gen_mul(10)
    src = T.codegen_enum_source(T.EN_VERIFY, p, None, T.Spec(p, "p = a * b"), 1)
    assert "#define TC_PERMUTED 1" in src
    L = host_words(src + "\nunsigned long long tc_host_unperm(unsigned long long y) "
                         "{ return tc_unperm(y); }\n")
    L.tc_host_unperm.restype = C.c_uint64
    L.tc_host_unperm.argtypes = [C.c_uint64]
    seen = set()
    for y in range(1 << 15):
        x = L.tc_host_unperm(y)
        assert x >> 15 == 0
        seen.add(x)
    assert len(seen) == 1 << 15
    for y in (1 << 15, 5 << 15 | 12345, (1 << 20) - 1):
        assert L.tc_host_unperm(y) >> 15 == y >> 15


def test_no_inputs_on_host():
    """A program without inputs has one assignment, 0: the generated code, run on the host, gives
    the reference's results (its --raw lines: verify "y = 0" one hit, "y = 1" none, search
    "y = 1" one hit, equivalence with a program whose z differs one hit)."""
    p = T.Program.from_asm(".out y z\nNAND ZERO\nSTO y\nNAND ONE\nSTO z\n")
    q = T.Program.from_asm(".out y z\nNAND ZERO\nSTO y\nSTO z\n")
    assert emulate(T.EN_VERIFY, p, None, T.Spec(p, "y = 0"), {"ticks": 1}) == (1, [0])
    assert emulate(T.EN_VERIFY, p, None, T.Spec(p, "y = 1"), {"ticks": 1}) == (0, [])
    assert emulate(T.EN_SEARCH, p, None, T.Spec(p, "y = 1", False), {"ticks": 1}) == (1, [0])
    assert emulate(T.EN_EQUIV, p, q, None, {"ticks": 1}) == (1, [0])
