"""Writes tests/golden/super.json from the reference's own superoptimizer front end.

    python tests/golden/make_super_golden.py

Needs the reference's library built from its sources (oracle/_ref/libalpha.so; oracle/Makefile
builds it on an x86 host that has the sources).  Every text of tests/super_cases.py is parsed by
the reference's super_parse; for each one it accepts, random programs are checked by its
super_check.

Also, for each specification of super_cases.SEARCHED, the shortest program the reference's
super_search finds and the check verdicts of it and of single-edit mutants of it.

Output: for each text "S:<sha256 of the parsed SuperSpec, 24 hex digits>" or "E:<error>"; the
verdicts ("1" passes, "0" fails; one character each) of the random programs of the accepted texts, in order
(the programs are regenerated from super_cases.program with seed 11); and the searched programs
with their mutants' verdicts (mutants regenerated with seed 12).
"""
from __future__ import annotations

import ctypes as C
import hashlib
import json
import os
import random
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

import oracle as O  # noqa: E402
import super_cases as SC  # noqa: E402
import tesseract_gb300 as T  # noqa: E402

N_TEXTS = 3000
PROGRAMS_PER_SPEC = 6
MUTANTS = 60


def ref_fns():
    R = O.ref_lib()
    R.super_parse.restype = C.c_int
    R.super_parse.argtypes = [C.c_char_p, C.POINTER(T.SuperSpec), C.c_char_p, C.c_size_t]
    R.super_check.restype = C.c_int
    R.super_check.argtypes = [C.POINTER(T.SuperSpec), C.POINTER(T.SuperProg), C.c_char_p,
                              C.c_size_t]
    return R


def to_prog(code):
    p = T.SuperProg()
    p.len = len(code)
    for i, (op, cell) in enumerate(code):
        p.code[i].op = op
        p.code[i].cell = cell.encode()
    return p


def cells_of(sp):
    return [sp.cell[i].name.decode() for i in range(sp.ncells)]


def verdict(R, sp, code):
    err = C.create_string_buffer(256)
    ok = R.super_check(C.byref(sp), C.byref(to_prog(code)), err, len(err))
    return "1" if ok else "0"


def main():
    R = ref_fns()
    R.super_search.argtypes = [C.POINTER(T.SuperSpec), C.POINTER(T.SuperOpts),
                               C.POINTER(T.SuperResult)]
    rng = random.Random(11)
    parsed, random_checks = [], []
    for text in SC.spec_texts(N_TEXTS):
        sp, err = T.SuperSpec(), C.create_string_buffer(256)
        if not R.super_parse(text.encode(), C.byref(sp), err, len(err)):
            parsed.append("E:" + err.value.decode())
            continue
        parsed.append("S:" + hashlib.sha256(bytes(sp)).hexdigest()[:24])
        for _ in range(PROGRAMS_PER_SPEC):
            random_checks.append(verdict(R, sp, SC.program(rng, cells_of(sp))))
    searched = []
    mrng = random.Random(12)
    for text in SC.SEARCHED:
        sp, err = T.SuperSpec(), C.create_string_buffer(256)
        assert R.super_parse(text.encode(), C.byref(sp), err, len(err)), (text, err.value)
        res = T.SuperResult()
        R.super_search(C.byref(sp), C.byref(T.SuperOpts(0, 0, 1, 16, 1)), C.byref(res))
        assert res.found, text
        code = [(res.prog.code[i].op, res.prog.code[i].cell.decode()) for i in range(res.prog.len)]
        progs = [code] + SC.mutants(mrng, code, cells_of(sp), MUTANTS)
        searched.append({"spec": text, "program": " ".join(("S:" if op else "") + c
                                                           for op, c in code),
                         "verdicts": [verdict(R, sp, c) for c in progs]})
    with open(os.path.join(HERE, "super.json"), "w") as f:
        json.dump({"n": N_TEXTS, "per_spec": PROGRAMS_PER_SPEC, "parsed": parsed,
                   "random_checks": "".join(random_checks), "mutants": MUTANTS,
                   "searched": [dict(s, verdicts="".join(s["verdicts"])) for s in searched]},
                  f, indent=0)
        f.write("\n")
    allv = random_checks + [v for s in searched for v in s["verdicts"]]
    print("wrote", len(parsed), "texts,", sum(p.startswith("S:") for p in parsed), "parsed,",
          len(allv), "checks,", sum(v == "1" for v in allv), "passing")


if __name__ == "__main__":
    main()
