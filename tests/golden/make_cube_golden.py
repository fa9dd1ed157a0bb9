"""Writes tests/golden/cube512.json.gz: the reference's own 512-machine cube demo programs, the
ones `alpha cube` runs (src/cubedemo.c:344-378), as the reference assembles them, and its
collectives across groups (a bitonic sort of lib/cube.inc's macros, gen_rank).

    python tests/golden/make_cube_golden.py

Needs the reference's sources (recorded by oracle/Makefile in oracle/_ref/SOURCE) and its library
built from them (oracle/_ref/libalpha.so).  Each demo whose program is assembly (any, rank, max,
sort, pack, perm, anf, ring) is taken from the demo table of src/cubedemo.c, assembled by the
reference's asm_string with its lib/std.inc and lib/cube.inc as `alpha cube` does
(src/cubedemo.c:676-682), and printed as a flat program listing (cells, links, instructions) by
this engine's printer, the macros' local cells (@<call>:<name>, which a listing outside a macro
cannot name) renamed mac<call>_<name>.  With each listing goes the digest of the reference's
program structure (tests/cases.py program_digest, by cell names: instructions, id and link cells,
inputs, outputs), which the listing must reassemble to; a listing numbers its cells in the order
it declares them, so only the names pin the cells.  tests/test_cube_ref_demos*.py run them."""
from __future__ import annotations

import ctypes as C
import gzip
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

sys.path.insert(0, os.path.dirname(HERE))

import oracle as O  # noqa: E402
import tesseract_gb300 as T  # noqa: E402
from cases import program_digest  # noqa: E402


def c_strings(text: str) -> list[str]:
    """The C string literals of an initializer, adjacent literals joined, escapes decoded."""
    out, i, cur, in_lit = [], 0, None, False
    while i < len(text):
        ch = text[i]
        if ch == '"':
            j, buf = i + 1, []
            while text[j] != '"':
                if text[j] == "\\":
                    buf.append({"n": "\n", "t": "\t", '"': '"', "\\": "\\"}[text[j + 1]])
                    j += 2
                else:
                    buf.append(text[j])
                    j += 1
            cur = (cur or "") + "".join(buf)
            i = j + 1
            continue
        if ch == "," and cur is not None:
            out.append(cur)
            cur = None
        elif ch not in " \t\n" and cur is not None:
            out.append(cur)
            cur = None
        elif ch not in " \t\n,":
            m = re.match(r"NULL", text[i:])
            if m:
                out.append(None)
                i += 4
                continue
        i += 1
    if cur is not None:
        out.append(cur)
    return out


LOCAL = r"@(\d+):(\w+)"  # a macro-local cell: @<call>:<name>


def print_program(p) -> str:
    """This engine's listing of a Program struct (tc_program_print)."""
    L = T.lib()
    n = L.tc_program_print(C.byref(p), None, 0)
    buf = C.create_string_buffer(n + 1)
    L.tc_program_print(C.byref(p), buf, n + 1)
    return buf.value.decode()


def add(out, name, what, p, R):
    listing = re.sub(LOCAL, r"mac\1_\2", print_program(p))
    digest = program_digest(p, lambda n: re.sub(LOCAL, r"mac\1_\2", n))
    R.program_free(C.byref(p))
    out[name] = {"what": what, "program": listing, "structure": digest}
    print(name, len(listing.splitlines()), "lines")


def demos(src: str):
    block = src[src.index("static const Demo demos[] = {"):]
    block = block[:block.index("};")]
    for entry in re.findall(r"\{(\"[a-z]+\".*?)\}", block, re.S):
        fields = c_strings(entry)
        yield fields[0], fields[1], fields[2]


def main():
    ref = O.reference_sources()
    R = O.ref_lib()
    lib = os.path.join(ref, "lib")
    with open(os.path.join(ref, "src", "cubedemo.c")) as f:
        table = list(demos(f.read()))
    out = {}
    for name, what, body in table:
        if body is None:
            continue  # made by a generator (walsh, xorconv, polymul, life)
        text = '.include "%s/std.inc"\n.include "%s/cube.inc"\n%s\n' % (lib, lib, body)
        p, err = T.ProgramStruct(), C.create_string_buffer(512)
        assert R.asm_string(text.encode(), name.encode(), b".", C.byref(p), err, len(err)), err.value
        add(out, name, what, p, R)
    # across groups: the bitonic sort from lib/cube.inc's compare-exchange macros (CMPX8 inside a
    # group, CMPX8_FAR across groups; stage st sorts blocks of 2^st machines up or down by bit st,
    # the last merge all up) at 1,024 and 2,048 machines, and the reference's gen_rank at 1,024
    # and 4,096 (the collectives of tests/test_cube.c:1130-1170)
    for dims in (10, 11):
        lines = ['.include "%s/std.inc"' % lib, '.include "%s/cube.inc"' % lib,
                 ".in v0 v1 v2 v3 v4 v5 v6 v7", ".out v0 v1 v2 v3 v4 v5 v6 v7"]
        for st in range(1, dims + 1):
            for j in range(st - 1, -1, -1):
                lines.append("%s v %d %s" % ("CMPX8" if j < 9 else "CMPX8_FAR", j,
                                             "ID%d" % st if st < dims else "ZERO"))
        p, err = T.ProgramStruct(), C.create_string_buffer(512)
        name = "sort%d" % dims
        assert R.asm_string(("\n".join(lines) + "\n").encode(), name.encode(), b".", C.byref(p),
                            err, len(err)), err.value
        add(out, name, "sort %d bytes across groups" % (1 << dims), p, R)
    R.gen_rank.argtypes = [C.POINTER(T.ProgramStruct), C.c_int]
    for dims in (10, 12):
        p = T.ProgramStruct()
        R.gen_rank(C.byref(p), dims)
        add(out, "rank%d" % dims, "gen_rank on %d machines" % (1 << dims), p, R)
    with gzip.open(os.path.join(HERE, "cube512.json.gz"), "wt") as f:
        json.dump(out, f, separators=(",", ":"))


if __name__ == "__main__":
    main()
