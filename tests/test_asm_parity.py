"""The assembler against the reference's own (src/asm.c), source by source.

Every source of tests/asm_cases.py must give the reference's result: the same Program (code,
cell numbering and names, inputs, outputs, cell kinds) or the same error message, including the
file:line and the macro call site.  On any host the first 3,000 are checked against
tests/golden/asm.json, which the reference wrote (tests/golden/make_asm_golden.py); where the
reference library is built here, 12,000 more are compared with it directly."""
import ctypes as C

import pytest

import asm_cases as AC
import oracle as O
import tesseract_gb300 as T
from cases import load


def assemble(src):
    p, err = T.ProgramStruct(), C.create_string_buffer(1024)
    if not T.lib().tc_asm_string(src.encode(), b"<src>", b".", C.byref(p), err, len(err)):
        return "E:" + err.value.decode()
    d = "P:" + AC.digest(p)
    T.lib().tc_program_free(C.byref(p))
    return d


@pytest.fixture
def include_dir(tmp_path, monkeypatch):
    AC.write_includes(str(tmp_path))
    monkeypatch.chdir(tmp_path)
    return tmp_path


def test_assembler_matches_reference_golden(include_dir):
    golden = load("asm.json")
    srcs = AC.cases(golden["n"])
    bad = [(s, g, m) for s, g in zip(srcs, golden["results"]) if (m := assemble(s)) != g]
    assert not bad, bad[:3]


@pytest.mark.skipif(not O.have_reference(), reason="the reference is not built here")
def test_assembler_matches_reference_live(include_dir):
    R = O.ref_lib()
    for src in AC.cases(12000, seed=4242):
        p, err = T.ProgramStruct(), C.create_string_buffer(1024)
        if R.asm_string(src.encode(), b"<src>", b".", C.byref(p), err, len(err)):
            want = "P:" + AC.digest(p)
            R.program_free(C.byref(p))
        else:
            want = "E:" + err.value.decode()
        assert assemble(src) == want, src


def test_file_entry_points(include_dir):
    """asm_file: relative includes from the file's own directory, text normalisation (UTF-8 and
    UTF-16 byte order marks), a missing file."""
    (include_dir / "sub" / "top.asm").write_text('.include "deep.inc"\nPICK s 3\n')
    p = T.Program.from_file(str(include_dir / "sub" / "top.asm"))
    assert p.names[2:] == ["deep", "s3", "ID3"]
    body = ".in a\nNAND a\nSTO b\n"
    for raw in (b"\xef\xbb\xbf" + body.encode(), b"\xff\xfe" + body.encode("utf-16-le"),
                b"\xfe\xff" + body.encode("utf-16-be")):
        (include_dir / "bom.asm").write_bytes(raw)
        q = T.Program.from_file(str(include_dir / "bom.asm"))
        assert q.names == ["ZERO", "ONE", "a", "b"] and len(q) == 2
    with pytest.raises(T.EngineError, match="cannot open file"):
        T.Program.from_file(str(include_dir / "absent.asm"))
