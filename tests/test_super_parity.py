"""The superoptimizer's front end against the reference's own (src/super.c:13-371, 900-1001).

Parser: every text of tests/super_cases.py gives the reference's SuperSpec byte for byte
(interchangeable inputs included) or its error message.  Check: random programs for every
accepted text, and the shortest programs the reference's own search found plus single-edit
mutants of them, get the reference's verdict.  The reference's check tries 16 random garbages per
sharing of cells and this one every garbage the program can observe, so the verdicts agree for
every program whose result does not hinge on rare garbage; the fixture has none that does.  On any
host the fixture tests/golden/super.json (tests/golden/make_super_golden.py) is the reference;
where its library is built here, 10,000 more texts are compared with it directly."""
import ctypes as C
import hashlib
import random

import pytest

import oracle as O
import super_cases as SC
import tesseract_gb300 as T
from cases import load


def parse(text):
    sp, err = T.SuperSpec(), C.create_string_buffer(256)
    L = T.lib()
    L.cuda_super_parse.restype = C.c_int
    L.cuda_super_parse.argtypes = [C.c_char_p, C.POINTER(T.SuperSpec), C.c_char_p, C.c_size_t]
    if not L.cuda_super_parse(text.encode(), C.byref(sp), err, len(err)):
        return "E:" + err.value.decode(), None
    return "S:" + hashlib.sha256(bytes(sp)).hexdigest()[:24], sp


def to_prog(code):
    p = T.SuperProg()
    p.len = len(code)
    for i, (op, cell) in enumerate(code):
        p.code[i].op = op
        p.code[i].cell = cell.encode()
    return p


def cells_of(sp):
    return [sp.cell[i].name.decode() for i in range(sp.ncells)]


def verdict(sp, code):
    return "1" if T.super_check(sp, to_prog(code))[0] else "0"


def test_parser_and_check_match_reference_golden():
    g = load("super.json")
    rng = random.Random(11)
    got_parsed, got_checks = [], []
    for text in SC.spec_texts(g["n"]):
        d, sp = parse(text)
        got_parsed.append(d)
        if sp is not None:
            for _ in range(g["per_spec"]):
                got_checks.append(verdict(sp, SC.program(rng, cells_of(sp))))
    bad = [(t, w, m) for t, w, m in zip(SC.spec_texts(g["n"]), g["parsed"], got_parsed) if w != m]
    assert not bad, bad[:5]
    assert "".join(got_checks) == g["random_checks"]


def test_check_on_searched_programs_and_mutants_matches_reference():
    g = load("super.json")
    mrng = random.Random(12)
    for s in g["searched"]:
        _, sp = parse(s["spec"])
        code = [(1, w[2:]) if w.startswith("S:") else (0, w) for w in s["program"].split()]
        progs = [code] + SC.mutants(mrng, code, cells_of(sp), g["mutants"])
        got = "".join(verdict(sp, c) for c in progs)
        assert got[0] == "1", s["spec"]  # the reference's shortest program passes
        assert got == s["verdicts"], (s["spec"], got, s["verdicts"])


@pytest.mark.skipif(not O.have_reference(), reason="the reference is not built here")
def test_parser_and_check_match_reference_live():
    R = O.ref_lib()
    R.super_parse.restype = C.c_int
    R.super_parse.argtypes = [C.c_char_p, C.POINTER(T.SuperSpec), C.c_char_p, C.c_size_t]
    R.super_check.restype = C.c_int
    R.super_check.argtypes = [C.POINTER(T.SuperSpec), C.POINTER(T.SuperProg), C.c_char_p,
                              C.c_size_t]
    rng = random.Random(3)
    for text in SC.spec_texts(13000, seed=99)[3000:]:
        ref, err = T.SuperSpec(), C.create_string_buffer(256)
        ok = R.super_parse(text.encode(), C.byref(ref), err, len(err))
        mine, sp = parse(text)
        if not ok:
            assert mine == "E:" + err.value.decode(), text
            continue
        assert sp is not None and bytes(sp) == bytes(ref), text
        for _ in range(3):
            code = SC.program(rng, cells_of(sp))
            want = R.super_check(C.byref(ref), C.byref(to_prog(code)), err, len(err))
            assert verdict(sp, code) == ("1" if want else "0"), (text, code, err.value)


def test_check_of_reads_before_writes():
    """A program that reads a scratch cell it never wrote is wrong for some garbage and
    rejected; RR's garbage before a NAND ZERO does not matter and the program passes."""
    _, sp = parse("RR = x")
    ok, why = T.super_check(sp, to_prog([(0, "ONE"), (0, "x"), (0, "_t1")]))
    assert not ok and "RR does not end" in why
    ok, _ = T.super_check(sp, to_prog([(0, "ZERO"), (0, "x"), (0, "ONE")]))
    assert ok
