"""Writes tests/golden/asm.json from the reference's own assembler.

    python tests/golden/make_asm_golden.py

Needs the reference's library built from its sources (oracle/_ref/libalpha.so; oracle/Makefile
builds it on an x86 host that has the sources).  Every source of tests/asm_cases.py is assembled
by the reference's asm_string in a scratch directory that holds the cases' include files, with
base directory ".", so that paths in error messages do not depend on the host.

Output, one entry per case in order: "P:<asm_cases.digest of the Program>" or "E:<error>".
"""
from __future__ import annotations

import ctypes as C
import json
import os
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

import asm_cases as AC  # noqa: E402
import oracle as O  # noqa: E402
import tesseract_gb300 as T  # noqa: E402

N_CASES = 3000


def reference_results(sources):
    R = O.ref_lib()
    out = []
    for src in sources:
        p, err = T.ProgramStruct(), C.create_string_buffer(1024)
        if R.asm_string(src.encode(), b"<src>", b".", C.byref(p), err, len(err)):
            out.append("P:" + AC.digest(p))
            R.program_free(C.byref(p))
        else:
            out.append("E:" + err.value.decode())
    return out


def main():
    sources = AC.cases(N_CASES)
    cwd = os.getcwd()
    with tempfile.TemporaryDirectory() as d:
        AC.write_includes(d)
        os.chdir(d)
        try:
            results = reference_results(sources)
        finally:
            os.chdir(cwd)
    with open(os.path.join(HERE, "asm.json"), "w") as f:
        json.dump({"n": N_CASES, "results": results}, f, indent=0)
        f.write("\n")
    print("wrote", len(results), "cases;", sum(r.startswith("P:") for r in results), "assembled")


if __name__ == "__main__":
    main()
