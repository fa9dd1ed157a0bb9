"""The superoptimizer's specification language against the reference's parser (src/super.c:
225-371): the parsed SuperSpec must be byte for byte the reference's."""
import ctypes as C
import os

import pytest

import oracle as O
import tesseract_gb300 as T

SPECS = ["RR = 1", "RR = !RR", "RR = 0", "RR = x", "RR = !x", "RR = RR & x", "RR = RR | x",
         "RR = !(RR | x)", "RR = RR & !x", "RR = RR | !x", "x = !RR; RR = RR",
         "dst = src; RR = src", "r = r | n", "r = r & n", "m = id & n", "o{x,y} = x & y",
         "o{x,y} = x | y", "RR = RR ^ x", "RR = !(RR ^ x)", "r = r ^ n", "o{x,y} = x ^ y",
         "r{a,b} = s ? a : b", "s{a,b} = a ^ b ^ c; c = a&b | a&c | b&c",
         "o{a0,a1} = s ? a1 : a0; ns := !s", "g = a & !b | a & g | !b & g",
         "p = p ^ (id & n); t = t ^ n", "r = (id ^ s) ? n : r"]
ERRORS = [("RR = ", "expected a name"), ("x = y; x = z", "set twice"),
          ("RR := x", "RR is set once"), ("a{a} = b", "must be another input"),
          ("q = a b", "unexpected")]


@pytest.mark.parametrize("text", SPECS)
def test_super_parse_matches_reference(text):
    mine = T.super_parse(text)
    if not O.have_reference():
        pytest.skip("the reference is not built here")
    R = O.ref_lib()
    R.super_parse.restype = C.c_int
    R.super_parse.argtypes = [C.c_char_p, C.POINTER(T.SuperSpec), C.c_char_p, C.c_size_t]
    ref, err = T.SuperSpec(), C.create_string_buffer(256)
    assert R.super_parse(text.encode(), C.byref(ref), err, len(err)), err.value
    assert bytes(mine) == bytes(ref)


@pytest.mark.parametrize("text,expect", ERRORS)
def test_super_parse_errors(text, expect):
    with pytest.raises(T.EngineError, match=expect):
        T.super_parse(text)


def test_super_check_of_the_reference_full_adder():
    """The 19-instruction full adder of tests/test_super.c:296-312 passes the check."""
    sp = T.super_parse("s{a,b} = a ^ b ^ c; c = a&b | a&c | b&c")
    code = ["NAND ZERO", "NAND a", "STO _t1", "NAND ONE", "NAND b", "STO _t2", "NAND b",
            "NAND _t1", "STO _t3", "NAND _t2", "NAND c", "STO _t4", "NAND c", "NAND _t2",
            "STO c", "NAND ONE", "NAND _t3", "NAND _t4", "STO s"]
    prog = T.SuperProg()
    prog.len = len(code)
    for i, line in enumerate(code):
        op, cell = line.split()
        prog.code[i].op = 1 if op == "STO" else 0
        prog.code[i].cell = cell.encode()
    ok, why = T.super_check(sp, prog)
    assert ok, why
    prog.code[17].cell = b"_t3"  # broken: reads the wrong scratch cell
    ok, why = T.super_check(sp, prog)
    assert not ok
