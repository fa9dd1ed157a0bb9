"""Writes tests/golden/spec.json from the reference's own specification code.

    python tests/golden/make_spec_golden.py

Needs the reference's library built from its sources (oracle/_ref/libalpha.so; oracle/Makefile
builds it on an x86 host that has the sources).  The program headers are assembled by the
reference's asm_string, every text of tests/spec_cases.py is parsed by its spec_parse, and every
vector name is resolved by its vec_resolve and printed by its vec_format.

Output, one entry per case in order:
    "S:<first 24 hex digits of the sha256 of the parsed struct's 14,744 bytes>" or "E:<error>"
and for each header the vec_resolve result of each name ([width, idx...]) and vec_format lines
for seeded bit values of its inputs and outputs.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

import oracle as O  # noqa: E402
import spec_cases as SC  # noqa: E402
import tesseract_gb300 as T  # noqa: E402

N_CASES = 2000
SPEC_BYTES = 14744  # sizeof the reference's struct Spec on LP64 (src/spec.c:20-29)


def digest(buf: bytes) -> str:
    import hashlib
    return hashlib.sha256(buf).hexdigest()[:24]


def ref_program(R, header):
    p, err = T.ProgramStruct(), C.create_string_buffer(512)
    assert R.asm_string(header.encode(), b"<spec>", b".", C.byref(p), err, len(err)), err.value
    return p


def main():
    R = O.ref_lib()
    R.vec_resolve.restype = C.c_int
    R.vec_resolve.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_char_p,
                              C.POINTER(C.c_int)]
    R.vec_format.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p, C.c_char_p,
                             C.c_size_t]
    progs = {h: ref_program(R, text) for h, text in SC.HEADERS.items()}
    results = []
    for h, text, inputs in SC.cases(N_CASES):
        err = C.create_string_buffer(512)
        s = R.spec_parse(text.encode(), C.byref(progs[h]), int(inputs), err, len(err))
        if s:
            results.append("S:" + digest(C.string_at(s, SPEC_BYTES)))
            R.spec_free(s)
        else:
            results.append("E:" + err.value.decode())
    vectors = {}
    for h, p in progs.items():
        good_in, bad_in, good_out, bad_out = SC.NAMES[h]
        names = sorted(set(good_in + bad_in + [o.strip() for x in good_out + bad_out
                                              for o in x.split(":") if o.strip()]))
        res = {}
        for which, lst, n in (("in", p.inputs, p.ninputs), ("out", p.outputs, p.noutputs)):
            for name in names:
                idx = (C.c_int * 64)()
                w = R.vec_resolve(C.byref(p), lst, n, name.encode(), idx)
                res[which + ":" + name] = [w] + [idx[i] for i in range(max(w, 0))]
            lines = []
            for seed in range(4):
                vals = (C.c_uint8 * n)(*[(seed * 7 + 3 * i + (i * i >> 2)) & 1 for i in range(n)])
                buf = C.create_string_buffer(4096)
                R.vec_format(C.byref(p), lst, n, vals, buf, len(buf))
                lines.append(buf.value.decode())
            res[which + ":format"] = lines
        vectors[h] = res
    out = {"n": N_CASES, "spec": results, "vectors": vectors}
    with open(os.path.join(HERE, "spec.json"), "w") as f:
        json.dump(out, f, indent=0)
        f.write("\n")
    print("wrote", len(results), "cases;",
          sum(r.startswith("S:") for r in results), "parsed")


if __name__ == "__main__":
    main()
