"""The bench's reference arm takes its inputs from the reference's own output, not from this
engine: the `gen mul --bits 16` text the reference printed (tests/golden/mul16.asm.gz, its sha256
pinned in programs.json) read by the oracle's loader, and the spec `p = a * b` laid out by the
oracle.  Both must equal what the engine builds, and running the arm's CPU enumerator must not
load the engine's library."""
import ctypes as C
import gzip
import hashlib
import os
import subprocess
import sys

import oracle as O
import tesseract_gb300 as T
from cases import GOLDEN, load

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def mul16_text():
    with gzip.open(os.path.join(GOLDEN, "mul16.asm.gz"), "rt") as f:
        return f.read()


def test_pinned_text_is_the_references():
    assert hashlib.sha256(mul16_text().encode()).hexdigest() == \
        load("programs.json")['mul:{"bits": 16}']


def test_oracle_inputs_equal_the_engines():
    p = O.PrintedProgram(mul16_text())
    mine = T.Program.gen_mul(16)
    assert p.s.len == len(mine) and p.s.ncells == mine.ncells
    # the same program; temporaries are numbered by first appearance in the text here and in
    # creation order by the generator, so instructions compare by cell name
    pn, mn = p.names, mine.names
    assert [(p.s.code[i].op, pn[p.s.code[i].addr]) for i in range(p.s.len)] == \
        [(op, mn[a]) for op, a in mine.code]
    assert [pn[c] for c in p.inputs] == [mn[c] for c in mine.inputs]
    assert [pn[c] for c in p.outputs] == [mn[c] for c in mine.outputs]
    spec = p.product_spec()
    assert C.string_at(C.addressof(spec), C.sizeof(spec)) == \
        C.string_at(T.Spec(mine, "p = a * b").p, C.sizeof(spec))


def test_reference_arm_cpu_leg_loads_no_engine_code():
    code = ("import sys; sys.path.insert(0, %r); import bench; "
            "prog, spec = bench.reference_inputs(); import oracle as O; "
            "r = O.enum_run_struct(O.verify_struct(prog, spec), threads=2, limit_chunks=2); "
            "assert r['hits'] == 0 and r['tried'] == 65536, r; "
            "maps = open('/proc/self/maps').read(); "
            "assert 'libtesseract_gb300' not in maps; assert 'liboracle' in maps; print('ok')"
            % ROOT)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, cwd=ROOT)
    assert r.returncode == 0 and "ok" in r.stdout, r.stderr
