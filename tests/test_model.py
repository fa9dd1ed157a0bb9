"""The host program model against the reference: generators, assembler, specifications.

Generators are pinned by the sha256 of the reference's own `alpha gen`/`alpha random` output
(tests/golden/programs.json, made by tests/golden/make_golden.py); the assembler and the spec
parser are compared with the reference's functions directly where the reference was built from
its sources here (oracle/_ref/libalpha.so), and against its known-answer tests everywhere."""
import ctypes as C
import hashlib
import json
import os

import pytest

import oracle as O
import tesseract_gb300 as T
from cases import load

REFERENCE = O.reference_sources() or ""
needs_ref = pytest.mark.skipif(not (O.have_reference() and REFERENCE),
                               reason="the reference is not built here")


@pytest.mark.parametrize("key", sorted(load("programs.json")))
def test_generator_matches_reference_output(key):
    kind, params = key.split(":", 1)
    params = json.loads(params)
    if kind == "mul":
        p = T.Program.gen_mul(params["bits"])
    elif kind == "hash":
        p = T.Program.gen_hash(params["bits"], params["rounds"])
    elif kind == "life":
        p = T.Program.gen_life(params["size"], params["size"])
    else:
        p = T.Program.random(params["cells"], params["len"], params["seed"])
    assert hashlib.sha256(p.text().encode()).hexdigest() == load("programs.json")[key]


def test_mul16_shape():
    """The verify workload: gen mul --bits 16 is 6,040 instructions over 72 cells."""
    p = T.Program.gen_mul(16)
    assert len(p) == 6040 and p.ncells == 72
    assert len(p.inputs) == 32 and len(p.outputs) == 32
    code = p.code
    assert sum(1 for op, _ in code if op == T.OP_NAND) == 4373


def _ref_program_struct(fn, *args):
    s = T.ProgramStruct()
    fn(C.byref(s), *args)
    return s


def _same_program(mine: T.Program, ref: T.ProgramStruct):
    m = mine.s
    assert m.len == ref.len and m.ncells == ref.ncells
    assert m.ninputs == ref.ninputs and m.noutputs == ref.noutputs
    assert all(m.code[i].op == ref.code[i].op and m.code[i].addr == ref.code[i].addr
               for i in range(m.len))
    assert [m.cell_names[i] for i in range(m.ncells)] == \
        [ref.cell_names[i] for i in range(ref.ncells)]
    assert [m.inputs[i] for i in range(m.ninputs)] == [ref.inputs[i] for i in range(ref.ninputs)]
    assert [m.outputs[i] for i in range(m.noutputs)] == \
        [ref.outputs[i] for i in range(ref.noutputs)]
    assert bool(m.special) == bool(ref.special)
    if m.special:
        for i in range(m.ncells):
            a, b = m.special[i], ref.special[i]
            assert (a.kind, a.dim) == (b.kind, b.dim)
            if a.kind == T.CK_LINK:
                assert a.src == b.src


@needs_ref
@pytest.mark.parametrize("shape", [(32, 32, 8, 8), (8, 8, 0, 9), (4, 6, 5, 5), (3, 3, 1, 1),
                                   (5, 4, 3, 7)])
def test_life_cube_generator_matches_reference(shape):
    w, h, rb, cb = shape
    R = O.ref_lib()
    board = (C.c_uint32 * (w * h))()
    ref = _ref_program_struct(R.gen_life_cube, w, h, rb, cb, board)
    mine = T.Program.gen_life_cube(w, h, rb, cb)
    _same_program(mine, ref)
    assert mine.board == list(board)
    R.program_free(C.byref(ref))


@needs_ref
@pytest.mark.parametrize("name", sorted(f for f in os.listdir(os.path.join(REFERENCE, "examples"))
                                        if f.endswith(".asm")) if os.path.isdir(
                                            os.path.join(REFERENCE, "examples")) else [])
def test_assembler_matches_reference_on_examples(name):
    path = os.path.join(REFERENCE, "examples", name)
    R = O.ref_lib()
    ref, err = T.ProgramStruct(), C.create_string_buffer(512)
    assert R.asm_file(path.encode(), C.byref(ref), err, len(err)), err.value
    mine = T.Program.from_file(path)
    _same_program(mine, ref)
    R.program_free(C.byref(ref))


ASM_ERRORS = [  # the reference's assembler error tests (tests/test_ref.c:272-300)
    ("FOO x\n", "unknown instruction or macro 'FOO'"),
    ("STO ONE\n", "cannot store to constant cell"),
    ("NAND\n", "expects exactly one cell"),
    ("NAND a b\n", "expects exactly one cell"),
    ("NAND 1x\n", "not a valid cell name"),
    ("NAND @t\n", "only allowed inside macros"),
    (".in ONE\n", "constant cell"),
    (".in a a\n", "declared twice"),
    (".bogus\n", "unknown directive"),
    (".endm\n", ".endm without .macro"),
    (".macro M\nNAND a\n", "missing .endm"),
    (".macro M x\nNAND x\n.endm\nM\n", "expects 1 argument, got 0"),
    (".macro R\nR\n.endm\nR\n", "nested too deeply"),
    (".macro NAND\n.endm\n", "cannot redefine instruction"),
    (".macro M\n.endm\n.macro M\n.endm\n", "already defined"),
    (".macro M\n.macro N\n.endm\n.endm\n", "inside macros"),
    (".macro M x\nNAND x\n.endm\nM @y\n", "only allowed inside macros"),
    (".include \"no_such_file.inc\"\n", "cannot open include file"),
    ("NAND a\nNAND b\nFOO\n", "<test>:3:"),
    (".macro M\nFOO\n.endm\nNAND a\nM\n",
     "<test>:2: unknown instruction or macro 'FOO' (in macro called at <test>:5)"),
]


@pytest.mark.parametrize("src,expect", ASM_ERRORS)
def test_assembler_errors(src, expect):
    with pytest.raises(T.EngineError) as e:
        T.Program.from_asm(src, "<test>", ".")
    assert expect in str(e.value)


def test_assembler_misc():
    p = T.Program.from_asm(".macro T\nSTO @t\n.endm\nT\nT\n")
    assert p.ncells == 4 and p.code[0][1] != p.code[1][1]
    assert p.names[2] == "@1:t" and p.names[3] == "@2:t"
    p = T.Program.from_asm("nand A\nsto a ; comment\n")
    assert len(p) == 2 and p.ncells == 3 and p.code[0][1] == p.code[1][1]
    p = T.Program.from_asm(".in a, b\n.out b\n")
    assert p.inputs == [2, 3] and p.outputs == [3]
    p = T.Program.from_asm(".link y = x @ 3\n.link z=y@12\nNAND z\nNAND ID4\n")
    sp = p.special
    assert sp[p.names.index("z")][0] == T.CK_LINK and p.dims() == 13
    assert sp[p.names.index("ID4")][:2] == (T.CK_ID, 4)
    p = T.Program.from_asm(".macro X v d\nNAND v#d\nNAND ID#d\n.endm\nX sum 3\n")
    assert p.names[2:] == ["sum3", "ID3"]


def test_program_print_roundtrip():
    for p in (T.Program.gen_mul(5), T.Program.gen_life_cube(4, 4, 5, 5),
              T.Program.random_in(20, 9, 300, 4)):
        q = T.Program.from_asm(p.text())
        pn, qn = p.names, q.names  # cells may be numbered differently: compare by name
        assert [(op, pn[a]) for op, a in p.code] == [(op, qn[a]) for op, a in q.code]
        assert [pn[a] for a in p.inputs] == [qn[a] for a in q.inputs]
        assert [pn[a] for a in p.outputs] == [qn[a] for a in q.outputs]
        assert sorted(pn) == sorted(qn)


# ---- specifications -----------------------------------------------------------------------

ADDER_HEADER = (".in  a7 a6 a5 a4 a3 a2 a1 a0  b7 b6 b5 b4 b3 b2 b1 b0  c\n"
                ".out s7 s6 s5 s4 s3 s2 s1 s0  c\n")
SPEC_VALUES = [  # tests/test_work.c:190-205: x = a7..a0 b7..b0 c, a in the high bits
    ("c:s = a + b + c", (200 << 9) | (100 << 1) | 1, 301),
    ("s = a * 2 + b", (3 << 9) | (4 << 1), 10),
    ("s = (a + b) * 2", (3 << 9) | (4 << 1), 14),
    ("s = a - b", (3 << 9) | (4 << 1), 255),
    ("s = ~a & 0xf0 | b ^ 1", (0x0f << 9) | (0x02 << 1), 0xf3),
    ("s = 1 << 3 >> 1", 0, 4),
    ("c = -c", 1, 1),
]
SPEC_ERRORS = [  # tests/test_work.c:213-220
    ("q = a", "no output called q", True),
    ("s = z", "no input called z", True),
    ("s = a +", "ends too early", True),
    ("s = (a", "expected )", True),
    ("s a", "expected =", True),
    ("s = a", "must be a number", False),
]


@pytest.mark.parametrize("text,x,want", SPEC_VALUES)
def test_spec_values(text, x, want):
    p = T.Program.from_asm(ADDER_HEADER)
    s = T.Spec(p, text)
    assert s.value(x) == want
    assert O.spec_value(s, x) == want


@pytest.mark.parametrize("text,expect,inputs", SPEC_ERRORS)
def test_spec_errors(text, expect, inputs):
    p = T.Program.from_asm(ADDER_HEADER)
    with pytest.raises(T.EngineError) as e:
        T.Spec(p, text, inputs)
    assert expect in str(e.value)


SPEC_LAYOUT_BYTES = 14744  # sizeof the reference's struct Spec on LP64 (src/spec.c:20-29)


@needs_ref
@pytest.mark.parametrize("text", [t for t, _, _ in SPEC_VALUES] +
                         ["c:s = a * b ^ (a << 3) - ~b", "s = a >> (b & 7) | -c"])
def test_spec_struct_is_the_references(text):
    p = T.Program.from_asm(ADDER_HEADER)
    mine = T.Spec(p, text)
    R = O.ref_lib()
    err = C.create_string_buffer(256)
    ref = R.spec_parse(text.encode(), p.ptr, 1, err, len(err))
    assert ref
    assert C.string_at(mine.p, SPEC_LAYOUT_BYTES) == C.string_at(ref, SPEC_LAYOUT_BYTES)
    for x in (0, 1, 12345, 0x1ffff, 0xabcde & 0x1ffff):
        assert R.spec_value(ref, x) == mine.value(x)
    R.spec_free(ref)
