"""The PTX the engine writes directly for quick-start builds of equivalence and search jobs
(csrc/ptxgen.c) assembles for sm_103a with ptxas (no GPU needed): single kernels of every shape
the writer has (inputs on lane patterns, lane bits, step bits and chunk bits; inputs past word bit
31; chunk-invariant LUTs hoisted or not; an output that is a constant or an input), a module of
several kernels, and the refusals.  ptxas's register report is checked for spills.  Skipped where
ptxas is absent; the GPU tests run these kernels against the oracle."""
import os
import re
import shutil
import subprocess
import tempfile

import pytest

import tesseract_gb300 as T

PTXAS = shutil.which("ptxas") or ("/usr/local/cuda/bin/ptxas"
                                  if os.path.exists("/usr/local/cuda/bin/ptxas") else None)
pytestmark = pytest.mark.skipif(PTXAS is None, reason="ptxas not installed")


def assemble(ptx: str, opt: int = 0) -> str:
    d = tempfile.mkdtemp()
    path = os.path.join(d, "gen.ptx")
    with open(path, "w") as f:
        f.write(ptx)
    r = subprocess.run([PTXAS, "-arch=sm_103a", "-O%d" % opt, "-v", path, "-o",
                        os.path.join(d, "gen.cubin")], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    return r.stderr


def pair(cells, width, length, seed, mutate):
    a = T.Program.random_in(cells, width, length, seed)
    return (T.EN_EQUIV, a, a.rewrite(seed + 7, mutate), None)


def cases():
    hash16 = T.Program.gen_hash(16, 5)
    target = T.lib().tc_toyhash(12345, 16, 5)
    mul12 = T.Program.gen_mul(12)
    const_out = T.Program.from_asm(".in a b c\n.out o\nNAND ZERO\nSTO o\n")
    same_out = T.Program.from_asm(".in a b\n.out o\nNAND ONE\nNAND ONE\nNAND a\nSTO o\n")
    return [
        ("equiv 8 inputs", pair(12, 8, 200, 1, True)),
        ("equiv 14 inputs", pair(20, 14, 900, 2, False)),
        ("equiv 22 inputs mutated", pair(40, 22, 3000, 3, True)),
        ("equiv 28 inputs", pair(64, 28, 4000, 4, False)),
        ("equiv 40 inputs", pair(48, 40, 1500, 5, True)),
        ("search hash16", (T.EN_SEARCH, hash16, None, T.Spec(hash16, "h = %d" % target, False))),
        ("search mul12", (T.EN_SEARCH, mul12, None, T.Spec(mul12, "p = 391", False))),
        ("equiv constant output", (T.EN_EQUIV, const_out, const_out, None)),
        ("equiv output is an input", (T.EN_EQUIV, same_out, same_out, None)),
    ]


CASES = cases()


@pytest.mark.parametrize("job", [c[1] for c in CASES], ids=[c[0] for c in CASES])
def test_kernel_assembles_without_spills(job):
    ptx = T.codegen_ptx_source(*job)
    assert ".entry tc_enum(" in ptx
    for opt in (0, 3):
        log = assemble(ptx, opt)
        spills = re.findall(r"(\d+) bytes spill stores", log)
        assert spills and all(s == "0" for s in spills), log


def test_chunk_invariant_luts_run_before_the_steps():
    """A 22-input pair whose outputs depend on few inputs: the LUTs that do not read a step input
    are written between the chunk's base and the first step; a program of 10 inputs has no step
    inputs at all, so every LUT is hoisted and a step only compares."""
    ptx = T.codegen_ptx_source(*pair(40, 22, 3000, 3, True))
    chunk = ptx[ptx.index("$BASE:"):ptx.index("$STEP:")]
    step = ptx[ptx.index("$STEP:"):ptx.index("$LANE:")]
    assert chunk.count("lop3.b32") + step.count("lop3.b32") > 0
    small = T.codegen_ptx_source(*pair(12, 10, 400, 9, True))
    step = small[small.index("$STEP:"):small.index("$LANE:")]
    chunk = small[small.index("$BASE:"):small.index("$STEP:")]
    compares = step.count(", 0xf6;")
    assert compares >= 1 and step.count("lop3.b32") == compares
    assert chunk.count("lop3.b32") >= 1


def test_module_of_several_kernels_assembles():
    jobs = [c[1] for c in CASES[:4]] + [CASES[5][1]]
    ptx = T.codegen_ptx_module(jobs)
    for k in range(len(jobs)):
        assert ".entry tc_enum_%d(" % k in ptx
    assemble(ptx, 0)


def test_refusals():
    mul8 = T.Program.gen_mul(8)
    with pytest.raises(T.EngineError, match="equivalence and search"):
        T.codegen_ptx_source(T.EN_VERIFY, mul8, None, T.Spec(mul8, "p = a * b"))
    a = T.Program.random_in(12, 10, 100, 3)
    with pytest.raises(T.EngineError, match="equivalence and search"):
        T.codegen_ptx_module([(T.EN_EQUIV, a, a, None, 2)])


@pytest.mark.parametrize("job", [c[1] for c in CASES], ids=[c[0] for c in CASES])
def test_every_value_is_written_before_it_is_read(job):
    """In the text, every %v register a lop3 reads has been written above it (in the prologue,
    the chunk's part or earlier in the step): the split into a chunk's and a step's LUTs keeps
    the mapped order's dependences."""
    ptx = T.codegen_ptx_source(*job)
    written = set()
    for line in ptx.splitlines():
        m = re.match(r"\s*(mov\.b32|shr\.s32|lop3\.b32) %v(\d+), (.*);", line)
        if not m:
            continue
        if m.group(1) == "lop3.b32":
            for r in re.findall(r"%v(\d+)", m.group(3)):
                assert r in written, line
        written.add(m.group(2))
