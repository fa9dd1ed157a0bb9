"""ORACLE -- test infrastructure, not product code.

ctypes bindings of oracle/liboracle.so, the CPU restatement of the reference's semantics
(oracle/oracle.c), and of the reference itself where it was built from its sources
(oracle/_ref/libalpha.so, x86 hosts with the sources mounted).  Imported only by tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg.
"""
from __future__ import annotations

import ctypes as C
import os

import tesseract_gb300 as T

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_LIB = os.path.join(HERE, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libalpha.so")
REF_BIN = os.path.join(HERE, "_ref", "alpha")

_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_LIB):
            raise RuntimeError(f"{ORACLE_LIB} is missing: build first")
        L = C.CDLL(ORACLE_LIB)
        P = C.POINTER(T.ProgramStruct)
        L.orc_enum_run.restype = C.c_int
        L.orc_enum_run.argtypes = [C.POINTER(T.EnumStruct), C.POINTER(T.EnumResult), C.c_int,
                                   C.c_uint64, C.c_char_p, C.c_size_t]
        L.orc_enum_ref.restype = C.c_int
        L.orc_enum_ref.argtypes = [C.POINTER(T.EnumStruct), C.POINTER(T.EnumResult), C.c_char_p,
                                   C.c_size_t]
        L.orc_spec_value.restype = C.c_uint64
        L.orc_spec_value.argtypes = [C.c_void_p, C.c_uint64]
        L.orc_cube_new.restype = C.c_void_p
        L.orc_cube_new.argtypes = [P, C.c_uint]
        L.orc_cube_free.argtypes = [C.c_void_p]
        L.orc_cube_get.restype = C.c_uint8
        L.orc_cube_get.argtypes = [C.c_void_p, C.c_uint, C.c_uint32]
        L.orc_cube_set.argtypes = [C.c_void_p, C.c_uint, C.c_uint32, C.c_uint8]
        L.orc_cube_rr.restype = C.c_uint8
        L.orc_cube_rr.argtypes = [C.c_void_p, C.c_uint]
        L.orc_cube_set_rr.argtypes = [C.c_void_p, C.c_uint, C.c_uint8]
        L.orc_cube_step.argtypes = [C.c_void_p]
        L.orc_cube_tick.argtypes = [C.c_void_p]
        L.orc_check_state.argtypes = [C.c_void_p, C.c_uint64]
        L.orc_dims.restype = C.c_uint
        L.orc_dims.argtypes = [P]
        L.orc_life_scalar.argtypes = [C.POINTER(C.c_uint8), C.c_int, C.c_int]
        L.orc_life_words.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int]
        L.orc_toyhash.restype = C.c_uint64
        L.orc_toyhash.argtypes = [C.c_uint64, C.c_int, C.c_int]
        _lib = L
    return _lib


def enum_run(mode, a, b=None, spec=None, ticks=1, part=0, part_end=None, parts=1, threads=None,
             limit_chunks=0) -> dict:
    """The enumeration on the CPU oracle's bit-sliced engine (orc_enum_run)."""
    e = T.make_enum(mode, a, b, spec, ticks, part, part_end, parts)
    r, err = T.EnumResult(), C.create_string_buffer(1024)
    if not lib().orc_enum_run(C.byref(e), C.byref(r), threads or os.cpu_count() or 1,
                              limit_chunks, err, len(err)):
        raise T.EngineError(err.value.decode())
    return r.as_dict()


def enum_ref(mode, a, b=None, spec=None, ticks=1, part=0, part_end=None, parts=1) -> dict:
    """The enumeration on the reference machine, one assignment at a time (small inputs)."""
    e = T.make_enum(mode, a, b, spec, ticks, part, part_end, parts)
    r, err = T.EnumResult(), C.create_string_buffer(1024)
    if not lib().orc_enum_ref(C.byref(e), C.byref(r), err, len(err)):
        raise T.EngineError(err.value.decode())
    return r.as_dict()


def spec_value(spec, x: int) -> int:
    return lib().orc_spec_value(spec.p, x)


def life_scalar(board: bytearray, w: int, h: int) -> None:
    buf = (C.c_uint8 * (w * h)).from_buffer(board)
    lib().orc_life_scalar(buf, w, h)


def life_words(board, gens: int, threads=None):
    """Game of Life on a torus of packed rows (numpy uint64 array, rows x words, bit j of word k
    = column 64 k + j), in place, on host threads."""
    h, w64 = board.shape
    lib().orc_life_words(board.ctypes.data, w64, h, gens, threads or os.cpu_count() or 1)


def toyhash(x: int, bits: int, rounds: int) -> int:
    return lib().orc_toyhash(x, bits, rounds)


class RefCube:
    """The reference machine: a lockstep cube of `machines` one-byte-per-cell machines."""

    def __init__(self, program, machines: int):
        self.program = program
        self.machines = machines
        self.h = lib().orc_cube_new(program.ptr, machines)

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_cube_free(self.h)
            self.h = None

    def get(self, k, a):
        return lib().orc_cube_get(self.h, k, a)

    def set(self, k, a, v):
        lib().orc_cube_set(self.h, k, a, v)

    def rr(self, k):
        return lib().orc_cube_rr(self.h, k)

    def set_rr(self, k, v):
        lib().orc_cube_set_rr(self.h, k, v)

    def step(self):
        lib().orc_cube_step(self.h)

    def tick(self):
        lib().orc_cube_tick(self.h)

    def check_state(self, seed):
        lib().orc_check_state(self.h, seed)


# ---- the reference itself (only where built from its sources) ----------------------------

def have_reference() -> bool:
    return os.path.exists(REF_LIB) and os.path.exists(REF_BIN)


def reference_sources() -> str | None:
    """The reference's source tree that oracle/_ref was built from (oracle/Makefile records it
    in oracle/_ref/SOURCE), when it is still present on this host; else None."""
    rec = os.path.join(HERE, "_ref", "SOURCE")
    if not os.path.exists(rec):
        return None
    with open(rec) as f:
        path = f.read().strip()
    return path if os.path.isdir(os.path.join(path, "src")) else None


def ref_lib():
    global _ref
    if _ref is None:
        L = C.CDLL(REF_LIB)
        P = C.POINTER(T.ProgramStruct)
        L.asm_string.restype = C.c_int
        L.asm_string.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, P, C.c_char_p, C.c_size_t]
        L.asm_file.restype = C.c_int
        L.asm_file.argtypes = [C.c_char_p, P, C.c_char_p, C.c_size_t]
        L.program_free.argtypes = [P]
        L.gen_mul.argtypes = [P, C.c_int]
        L.gen_hash.restype = C.c_int
        L.gen_hash.argtypes = [P, C.c_int, C.c_int]
        L.gen_life_cube.argtypes = [P, C.c_int, C.c_int, C.c_int, C.c_int,
                                    C.POINTER(C.c_uint32)]
        L.gen_life.argtypes = [P, C.c_int, C.c_int, C.POINTER(C.c_uint32)]
        L.random_program.argtypes = [P, C.c_uint32, C.c_size_t, C.c_uint64]
        L.spec_parse.restype = C.c_void_p
        L.spec_parse.argtypes = [C.c_char_p, P, C.c_int, C.c_char_p, C.c_size_t]
        L.spec_value.restype = C.c_uint64
        L.spec_value.argtypes = [C.c_void_p, C.c_uint64]
        L.spec_free.argtypes = [C.c_void_p]
        L.enum_run.restype = C.c_int
        L.enum_run.argtypes = [C.POINTER(T.EnumStruct), C.POINTER(T.EnumResult), C.c_char_p,
                               C.c_size_t]
        _ref = L
    return _ref


# ---- inputs for the reference arm that need nothing of the product ------------------------

class _RefItem(C.Structure):
    _fields_ = [("op", C.c_int), ("v", C.c_uint64)]


class RefSpec(C.Structure):
    """The reference's private struct Spec (src/spec.c:20-29), filled in here for `p = a * b`
    shaped specifications without its parser or this engine's."""
    _fields_ = [("width", C.c_int), ("out", C.c_uint32 * 64), ("nvars", C.c_int),
                ("var_name", (C.c_char * 64) * 32), ("var_bits", C.c_int * 32),
                ("var_pos", (C.c_int * 64) * 32), ("rpn", _RefItem * 256), ("nrpn", C.c_int),
                ("depth", C.c_int), ("max_depth", C.c_int)]


_T_VAR, _T_MUL = 1, 4  # RPN items (src/spec.c:11)


class PrintedProgram:
    """A Program struct (the reference's layout) from the text its generators print (`alpha gen
    ...`, src/build.c:417-444): .in/.out lines and one NAND or STO per line, cells numbered ZERO,
    ONE, then by first appearance.  The printed form has no macros, includes or links."""

    def __init__(self, text: str):
        names, index, code, ins, outs = ["ZERO", "ONE"], {"zero": 0, "one": 1}, [], [], []

        def cell(n):
            if n.lower() not in index:
                index[n.lower()] = len(names)
                names.append(n)
            return index[n.lower()]
        for line in text.splitlines():
            f = line.split(";")[0].split()
            if not f:
                continue
            if f[0] in (".in", ".out"):
                (ins if f[0] == ".in" else outs).extend(cell(n) for n in f[1:])
            else:
                code.append((0 if f[0].upper() == "NAND" else 1, cell(f[1])))
        self.names, self.inputs, self.outputs = names, ins, outs
        self._code = (T.Instr * len(code))(*[T.Instr(op, a) for op, a in code])
        self._names = (C.c_char_p * len(names))(*[n.encode() for n in names])
        self._in = (C.c_uint32 * len(ins))(*ins)
        self._out = (C.c_uint32 * len(outs))(*outs)
        self.s = T.ProgramStruct(self._code, len(code), len(names), self._names, self._in,
                                 len(ins), self._out, len(outs), None)

    def vector(self, cells, stem):
        """Positions in `cells` of stem0, stem1, ... (bit order)."""
        pos = {self.names[c].lower(): i for i, c in enumerate(cells)}
        out = []
        while f"{stem}{len(out)}" in pos:
            out.append(pos[f"{stem}{len(out)}"])
        return out

    def product_spec(self, out="p", x="a", y="b") -> RefSpec:
        """`out = x * y` over the input vectors x and y (input k of n is bit n-1-k)."""
        s = RefSpec()
        n = len(self.inputs)
        for c in [self.outputs[i] for i in self.vector(self.outputs, out)]:
            s.out[s.width] = c
            s.width += 1
        for k, stem in enumerate((x, y)):
            bits = self.vector(self.inputs, stem)
            s.var_name[k].value = stem.encode()
            s.var_bits[k] = len(bits)
            for b, i in enumerate(bits):
                s.var_pos[k][b] = n - 1 - i
        s.nvars = 2
        for i, (op, v) in enumerate(((_T_VAR, 0), (_T_VAR, 1), (_T_MUL, 0))):
            s.rpn[i].op, s.rpn[i].v = op, v
        s.nrpn, s.depth, s.max_depth = 3, 1, 2
        return s


def verify_struct(prog: PrintedProgram, spec: RefSpec) -> "T.EnumStruct":
    e = T.EnumStruct()
    e.mode = T.EN_VERIFY
    e.a = C.pointer(prog.s)
    e.spec = C.cast(C.pointer(spec), C.c_void_p)
    e.ticks, e.part, e.part_end, e.parts = 1, 0, 0, 1
    return e


def enum_run_struct(e, threads=None, limit_chunks=0) -> dict:
    """orc_enum_run on a prepared Enum struct."""
    r, err = T.EnumResult(), C.create_string_buffer(1024)
    if not lib().orc_enum_run(C.byref(e), C.byref(r), threads or os.cpu_count() or 1,
                              limit_chunks, err, len(err)):
        raise T.EngineError(err.value.decode())
    return r.as_dict()
