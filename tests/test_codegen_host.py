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

import numpy as np
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
    space = 1 << len(a.inputs)
    words = (space + 31) // 32
    out = np.zeros(words, dtype=np.uint32)
    L.tc_host_words(0, words, out.ctypes.data)
    if space < 32:
        out &= np.uint32((1 << space) - 1)
    hits = int(sum(bin(int(w)).count("1") for w in out)) if words < 64 else \
        int(np.unpackbits(out.view(np.uint8)).sum())
    first = []
    for w in np.nonzero(out)[0]:
        v = int(out[w])
        while v and len(first) < 16:
            low = v & -v
            first.append(int(w) * 32 + low.bit_length() - 1)
            v ^= low
        if len(first) >= 16:
            break
    return hits, first


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
