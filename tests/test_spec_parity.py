"""The specification parser and the vector helpers against the reference's own (src/spec.c).

Every text of tests/spec_cases.py (well-formed, damaged, nested past the stack, too long) must
give the reference's result: the same parsed struct, byte for byte, or the same error message.
On any host the first 2,000 are checked against tests/golden/spec.json, which the reference
wrote (tests/golden/make_spec_golden.py); where the reference library is built here, 20,000 more
are compared with it directly.  vec_resolve and vec_format are checked the same way."""
import ctypes as C
import hashlib

import pytest

import oracle as O
import spec_cases as SC
import tesseract_gb300 as T
from cases import load

SPEC_BYTES = 14744  # sizeof the reference's struct Spec on LP64 (src/spec.c:20-29)

_programs = {}


def program(h):
    if h not in _programs:
        _programs[h] = T.Program.from_asm(SC.HEADERS[h])
    return _programs[h]


def parse(h, text, inputs):
    err = C.create_string_buffer(512)
    s = T.lib().cuda_spec_parse(text.encode(), program(h).ptr, int(inputs), err, len(err))
    if not s:
        return "E:" + err.value.decode(), None
    raw = C.string_at(s, SPEC_BYTES)
    T.lib().cuda_spec_free(s)
    return "S:" + hashlib.sha256(raw).hexdigest()[:24], raw


def test_parser_matches_reference_golden():
    golden = load("spec.json")
    cases = SC.cases(golden["n"])
    bad = [(c, g, parse(*c)[0]) for c, g in zip(cases, golden["spec"]) if parse(*c)[0] != g]
    assert not bad, bad[:5]


@pytest.mark.skipif(not O.have_reference(), reason="the reference is not built here")
def test_parser_matches_reference_live():
    R = O.ref_lib()
    refp = {}
    for h, text in SC.HEADERS.items():
        p, err = T.ProgramStruct(), C.create_string_buffer(512)
        assert R.asm_string(text.encode(), b"<spec>", b".", C.byref(p), err, len(err))
        refp[h] = p
    for h, text, inputs in SC.cases(22000, seed=77)[2000:]:
        mine, raw = parse(h, text, inputs)
        err = C.create_string_buffer(512)
        s = R.spec_parse(text.encode(), C.byref(refp[h]), int(inputs), err, len(err))
        if s:
            theirs = C.string_at(s, SPEC_BYTES)
            for x in (0, 1, 0x5a5a5a5a5a5a5a5a, 2**64 - 1, 0x123456789abcdef):
                assert R.spec_value(s, x) == O.lib().orc_spec_value(s, x)
            R.spec_free(s)
            assert raw == theirs, (h, text)
        else:
            assert mine == "E:" + err.value.decode(), (h, text)


def test_values_of_parsed_specs_match_the_oracle():
    """cuda_spec_value (the host evaluator) against the oracle's, on every parsed case."""
    for h, text, inputs in SC.cases(2000):
        err = C.create_string_buffer(512)
        s = T.lib().cuda_spec_parse(text.encode(), program(h).ptr, int(inputs), err, len(err))
        if not s:
            continue
        for x in (0, 1, 0x1ffff, 0x5a5a5a5a5a5a5a5a, 2**64 - 1, 0x0123456789abcdef):
            assert T.lib().cuda_spec_value(s, x) == O.lib().orc_spec_value(s, x), (text, x)
        T.lib().cuda_spec_free(s)


def test_vectors_match_reference_golden():
    golden = load("spec.json")["vectors"]
    L = T.lib()
    L.tc_vec_resolve.restype = C.c_int
    L.tc_vec_resolve.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_char_p,
                                 C.POINTER(C.c_int)]
    L.tc_vec_format.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p, C.c_char_p,
                                C.c_size_t]
    for h, want in golden.items():
        p = program(h)
        s = p.s
        for which, lst, n in (("in", s.inputs, s.ninputs), ("out", s.outputs, s.noutputs)):
            for key, res in want.items():
                kind, name = key.split(":", 1)
                if kind != which or name == "format":
                    continue
                idx = (C.c_int * 64)()
                w = L.tc_vec_resolve(p.ptr, lst, n, name.encode(), idx)
                assert [w] + [idx[i] for i in range(max(w, 0))] == res, (h, key)
            for seed, line in enumerate(want[which + ":format"]):
                vals = (C.c_uint8 * n)(*[(seed * 7 + 3 * i + (i * i >> 2)) & 1 for i in range(n)])
                buf = C.create_string_buffer(4096)
                L.tc_vec_format(p.ptr, lst, n, vals, buf, len(buf))
                assert buf.value.decode() == line, (h, which, seed)
