"""Python bindings of the GB300 engine for Tesseract's bit-sliced NAND/STO machine.

The engine itself is C and CUDA behind a C ABI (include/tesseract_cuda.h,
include/tesseract_model.h) in ``libtesseract_gb300.so``; this module binds it with ctypes and
mirrors the reference's host interface for the hot path:

    Program            src/isa.h Program, built by the assembler or the generators
    Spec               spec_parse / spec_value (src/spec.h)
    enum_run           enum_run (src/enum.h:37): verify / equiv / search
    check              check_lanes (src/check.h:25) with the CUDA engine
    Cube               LaneCube + jit_cube_run (src/lanes.h, src/jit.h)

There is no CPU fallback: when the shared library is missing every call raises.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libtesseract_gb300.so")

EN_VERIFY, EN_EQUIV, EN_SEARCH = 0, 1, 2
EN_SHOW = 16
OP_NAND, OP_STO = 0, 1
CK_PLAIN, CK_ID, CK_LINK = 0, 1, 2


class Instr(C.Structure):
    _fields_ = [("op", C.c_uint8), ("addr", C.c_uint32)]


class CellInfo(C.Structure):
    _fields_ = [("kind", C.c_uint8), ("dim", C.c_uint8), ("src", C.c_uint32)]


class ProgramStruct(C.Structure):
    _fields_ = [("code", C.POINTER(Instr)), ("len", C.c_size_t), ("ncells", C.c_uint32),
                ("cell_names", C.POINTER(C.c_char_p)), ("inputs", C.POINTER(C.c_uint32)),
                ("ninputs", C.c_size_t), ("outputs", C.POINTER(C.c_uint32)),
                ("noutputs", C.c_size_t), ("special", C.POINTER(CellInfo))]


class EnumStruct(C.Structure):
    _fields_ = [("mode", C.c_int), ("a", C.POINTER(ProgramStruct)),
                ("b", C.POINTER(ProgramStruct)), ("spec", C.c_void_p), ("ticks", C.c_uint),
                ("threads", C.c_int), ("idle", C.c_int), ("excluded", C.c_void_p),
                ("part", C.c_int), ("part_end", C.c_int), ("parts", C.c_int)]


class EnumResult(C.Structure):
    _fields_ = [("space", C.c_uint64), ("tried", C.c_uint64), ("hits", C.c_uint64),
                ("hit", C.c_uint64 * EN_SHOW), ("nhit", C.c_int), ("seconds", C.c_double),
                ("ops", C.c_uint64), ("threads", C.c_int)]

    def as_dict(self):
        return {"space": self.space, "tried": self.tried, "hits": self.hits,
                "hit": list(self.hit[: self.nhit]), "ops": self.ops,
                "seconds": self.seconds, "threads": self.threads}


class CheckResult(C.Structure):
    _fields_ = [("ok", C.c_int), ("compared", C.c_uint64), ("tick", C.c_uint64),
                ("pc", C.c_long), ("lane", C.c_uint), ("cell", C.c_long), ("want", C.c_uint),
                ("got", C.c_uint)]


SUPER_CELLS, SUPER_LEN, SUPER_NAME = 16, 64, 24


class SuperCell(C.Structure):
    _fields_ = [("name", C.c_char * SUPER_NAME), ("in_", C.c_int), ("out", C.c_int),
                ("init", C.c_uint64), ("target", C.c_uint64), ("alias", C.c_uint32),
                ("sym_prev", C.c_int)]


class SuperSpec(C.Structure):
    _fields_ = [("nvars", C.c_int), ("mask", C.c_uint64), ("rr_in", C.c_int), ("rr_out", C.c_int),
                ("rr_target", C.c_uint64), ("ncells", C.c_int),
                ("cell", SuperCell * SUPER_CELLS)]


class SuperInstr(C.Structure):
    _fields_ = [("op", C.c_uint8), ("cell", C.c_char * SUPER_NAME)]


class SuperProg(C.Structure):
    _fields_ = [("len", C.c_int), ("code", SuperInstr * SUPER_LEN)]


class SuperOpts(C.Structure):
    _fields_ = [("threads", C.c_int), ("part", C.c_int), ("parts", C.c_int), ("max_cost", C.c_int),
                ("quiet", C.c_int)]


class SuperResult(C.Structure):
    _fields_ = [("found", C.c_int), ("cost", C.c_int), ("below", C.c_int),
                ("contradiction", C.c_int), ("prog", SuperProg), ("nodes", C.c_uint64),
                ("seconds", C.c_double)]


class LaunchStats(C.Structure):
    _fields_ = [("kernel_ms", C.c_double), ("regs", C.c_int), ("local_bytes", C.c_int),
                ("grid", C.c_uint), ("block", C.c_uint), ("compile_seconds", C.c_double),
                ("cached", C.c_int), ("luts_per_step", C.c_int), ("luts_per_stretch", C.c_int),
                ("stretch_steps", C.c_int), ("compare_ops", C.c_int),
                ("logic_ops_per_word", C.c_double), ("ptx", C.c_int)]


_lib = None


class EngineError(RuntimeError):
    pass


def lib():
    """The shared library, loaded once.  Raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise EngineError(f"{LIB_PATH} is missing: run tesseract_gb300.build.build() first")
        L = C.CDLL(LIB_PATH)
        P = C.POINTER(ProgramStruct)
        sig = {
            "tc_program_free": (None, [P]),
            "tc_program_print": (C.c_size_t, [P, C.c_char_p, C.c_size_t]),
            "tc_program_copy": (C.c_int, [P, P]),
            "tc_program_dims": (C.c_uint, [P]),
            "tc_asm_string": (C.c_int, [C.c_char_p, C.c_char_p, C.c_char_p, P, C.c_char_p,
                                        C.c_size_t]),
            "tc_asm_file": (C.c_int, [C.c_char_p, P, C.c_char_p, C.c_size_t]),
            "tc_gen_mul": (None, [P, C.c_int]),
            "tc_gen_hash": (C.c_int, [P, C.c_int, C.c_int]),
            "tc_toyhash": (C.c_uint64, [C.c_uint64, C.c_int, C.c_int]),
            "tc_gen_life": (None, [P, C.c_int, C.c_int, C.POINTER(C.c_uint32)]),
            "tc_gen_life_cube": (None, [P, C.c_int, C.c_int, C.c_int, C.c_int,
                                        C.POINTER(C.c_uint32)]),
            "tc_grid_machine": (C.c_uint, [C.c_uint, C.c_uint, C.c_int]),
            "tc_random_program": (None, [P, C.c_uint32, C.c_size_t, C.c_uint64]),
            "tc_random_program_in": (None, [P, C.c_uint32, C.c_uint32, C.c_size_t, C.c_uint64]),
            "tc_rewrite_program": (None, [P, P, C.c_uint64, C.c_int]),
            "cuda_spec_parse": (C.c_void_p, [P, C.c_int, C.c_char_p, C.c_size_t]),
            "cuda_spec_free": (None, [C.c_void_p]),
            "cuda_spec_width": (C.c_int, [C.c_void_p]),
            "cuda_spec_out_cell": (C.c_uint32, [C.c_void_p, C.c_int]),
            "cuda_spec_value": (C.c_uint64, [C.c_void_p, C.c_uint64]),
            "cuda_engine_init": (C.c_int, [C.c_int, C.c_char_p, C.c_size_t]),
            "cuda_device_info": (C.c_int, [C.c_char_p, C.c_size_t]),
            "cuda_enum_run": (C.c_int, [C.POINTER(EnumStruct), C.POINTER(EnumResult), C.c_char_p,
                                        C.c_size_t]),
            "tc_codegen_enum": (C.c_void_p, [C.c_void_p, C.POINTER(C.c_size_t)]),
            "cuda_last_launch": (C.c_int, [C.POINTER(LaunchStats)]),
            "cuda_check": (C.c_int, [P, C.c_uint64, C.c_uint, C.POINTER(CheckResult),
                                     C.c_char_p, C.c_size_t]),
            "cuda_cube_new": (C.c_int, [P, C.POINTER(C.c_void_p), C.c_char_p, C.c_size_t]),
            "cuda_cube_free": (None, [C.c_void_p]),
            "cuda_cube_groups": (C.c_uint, [C.c_void_p]),
            "cuda_cube_segments": (C.c_uint, [C.c_void_p]),
            "cuda_cube_kernels": (C.c_uint, [C.c_void_p]),
            "cuda_cube_closing_copies": (C.c_uint, [C.c_void_p]),
            "cuda_cube_load": (C.c_int, [C.c_void_p, C.c_uint, C.c_void_p, C.c_void_p,
                                         C.c_char_p, C.c_size_t]),
            "cuda_cube_store": (C.c_int, [C.c_void_p, C.c_uint, C.c_void_p, C.c_void_p,
                                          C.c_char_p, C.c_size_t]),
            "cuda_cube_read_words": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_char_p,
                                               C.c_size_t]),
            "cuda_cube_write_words": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_char_p,
                                                C.c_size_t]),
            "cuda_cube_run": (C.c_int, [C.c_void_p, C.c_uint64, C.c_char_p, C.c_size_t]),
            "cuda_lop3_peak": (C.c_int, [C.POINTER(C.c_double), C.POINTER(C.c_double),
                                         C.c_char_p, C.c_size_t]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        # cuda_spec_parse takes the text first
        L.cuda_spec_parse.argtypes = [C.c_char_p, P, C.c_int, C.c_char_p, C.c_size_t]
        _lib = L
    return _lib


def _err():
    return C.create_string_buffer(1024)


class Program:
    """A NAND/STO program owned by the engine's library (src/isa.h Program)."""

    def __init__(self):
        self.s = ProgramStruct()
        self._owned = False

    def __del__(self):
        if getattr(self, "_owned", False) and _lib is not None:
            _lib.tc_program_free(C.byref(self.s))
            self._owned = False

    @property
    def ptr(self):
        return C.pointer(self.s)

    # ---- construction -------------------------------------------------------------------
    @classmethod
    def _made(cls, fn, *args):
        p = cls()
        fn(C.byref(p.s), *args)
        p._owned = True
        return p

    @classmethod
    def from_asm(cls, text: str, name: str = "<string>", base_dir: str = "."):
        p, e = cls(), _err()
        if not lib().tc_asm_string(text.encode(), name.encode(), base_dir.encode(),
                                   C.byref(p.s), e, len(e)):
            raise EngineError(e.value.decode())
        p._owned = True
        return p

    @classmethod
    def from_file(cls, path: str):
        p, e = cls(), _err()
        if not lib().tc_asm_file(path.encode(), C.byref(p.s), e, len(e)):
            raise EngineError(e.value.decode())
        p._owned = True
        return p

    @classmethod
    def gen_mul(cls, bits: int):
        return cls._made(lib().tc_gen_mul, bits)

    @classmethod
    def gen_hash(cls, bits: int, rounds: int):
        p = cls()
        if not lib().tc_gen_hash(C.byref(p.s), bits, rounds):
            raise EngineError(f"no toy hash for {bits} bits")
        p._owned = True
        return p

    @classmethod
    def gen_life(cls, w: int, h: int):
        board = (C.c_uint32 * (w * h))()
        p = cls._made(lib().tc_gen_life, w, h, board)
        p.board = list(board)
        return p

    @classmethod
    def gen_life_cube(cls, w: int, h: int, rbits: int, cbits: int):
        board = (C.c_uint32 * (w * h))()
        p = cls._made(lib().tc_gen_life_cube, w, h, rbits, cbits, board)
        p.board = list(board)
        return p

    @classmethod
    def random(cls, cells: int, length: int, seed: int):
        return cls._made(lib().tc_random_program, cells, length, seed)

    @classmethod
    def gen_cube_demo(cls, name: str, dims: int):
        """The cube demo `name` (any, rank, sort, max, pack, anf, walsh, xorconv, ring, polymul)
        for 2^dims machines."""
        fn = {"any": "tc_gen_cube_any", "rank": "tc_gen_cube_rank", "sort": "tc_gen_cube_sort",
              "max": "tc_gen_cube_max", "pack": "tc_gen_cube_pack", "anf": "tc_gen_cube_anf",
              "walsh": "tc_gen_cube_walsh", "xorconv": "tc_gen_cube_xorconv",
              "ring": "tc_gen_cube_ring", "polymul": "tc_gen_cube_polymul"}
        p = cls()
        f = getattr(lib(), fn[name])
        f.argtypes = [C.POINTER(ProgramStruct), C.c_int]
        f.restype = None
        f(C.byref(p.s), dims)
        return p

    @classmethod
    def random_in(cls, cells: int, width: int, length: int, seed: int):
        return cls._made(lib().tc_random_program_in, cells, width, length, seed)

    def rewrite(self, seed: int, mutate: bool = False):
        p = Program()
        lib().tc_rewrite_program(self.ptr, C.byref(p.s), seed, int(mutate))
        p._owned = True
        return p

    # ---- views --------------------------------------------------------------------------
    def text(self) -> str:
        n = lib().tc_program_print(self.ptr, None, 0)
        buf = C.create_string_buffer(n + 1)
        lib().tc_program_print(self.ptr, buf, n + 1)
        return buf.value.decode()

    def __len__(self):
        return self.s.len

    @property
    def ncells(self):
        return self.s.ncells

    @property
    def names(self):
        return [self.s.cell_names[i].decode() for i in range(self.s.ncells)]

    @property
    def inputs(self):
        return [self.s.inputs[i] for i in range(self.s.ninputs)]

    @property
    def outputs(self):
        return [self.s.outputs[i] for i in range(self.s.noutputs)]

    @property
    def code(self):
        return [(self.s.code[i].op, self.s.code[i].addr) for i in range(self.s.len)]

    @property
    def special(self):
        if not self.s.special:
            return None
        return [(self.s.special[i].kind, self.s.special[i].dim, self.s.special[i].src)
                for i in range(self.s.ncells)]

    def dims(self):
        return lib().tc_program_dims(self.ptr)


class Spec:
    """A specification parsed against a program (spec_parse, src/spec.c:272-327)."""

    def __init__(self, program: Program, text: str, inputs_allowed: bool = True):
        e = _err()
        self.program = program
        self.text = text
        self.p = lib().cuda_spec_parse(text.encode(), program.ptr, int(inputs_allowed), e,
                                       len(e))
        if not self.p:
            raise EngineError(e.value.decode())

    def __del__(self):
        if getattr(self, "p", None) and _lib is not None:
            _lib.cuda_spec_free(self.p)
            self.p = None

    @property
    def width(self):
        return lib().cuda_spec_width(self.p)

    def out_cell(self, bit: int):
        return lib().cuda_spec_out_cell(self.p, bit)

    def value(self, x: int):
        return lib().cuda_spec_value(self.p, x)


def make_enum(mode, a: Program, b: Program | None = None, spec: Spec | None = None, ticks=1,
              part=0, part_end=None, parts=1) -> EnumStruct:
    e = EnumStruct()
    e.mode = mode
    e.a = a.ptr
    e.b = b.ptr if b is not None else C.POINTER(ProgramStruct)()
    e.spec = spec.p if spec is not None else None
    e.ticks = ticks
    e.part = part
    e.part_end = part if part_end is None else part_end
    e.parts = parts
    return e


def enum_run(mode, a: Program, b: Program | None = None, spec: Spec | None = None, ticks=1,
             part=0, part_end=None, parts=1) -> dict:
    """verify / equiv / search on the GPU (cuda_enum_run)."""
    e = make_enum(mode, a, b, spec, ticks, part, part_end, parts)
    r, err = EnumResult(), _err()
    if not lib().cuda_enum_run(C.byref(e), C.byref(r), err, len(err)):
        raise EngineError(err.value.decode())
    return r.as_dict()


class _TuneCand(C.Structure):
    _fields_ = [("block", C.c_int), ("step_bits", C.c_int), ("ms", C.c_double)]


class CudaTune(C.Structure):
    _fields_ = [("n", C.c_int), ("ncand", C.c_int), ("best", C.c_int),
                ("cand", _TuneCand * 9), ("probe_fraction", C.c_double)]


def enum_tune(mode, a: Program, b: Program | None = None, spec: Spec | None = None, ticks=1,
              part=0, part_end=None, parts=1) -> dict:
    """The autotuner (cuda_enum_tune): the job's kernel variants timed on the job; the fastest
    becomes its kernel for every later launch in this process."""
    e = make_enum(mode, a, b, spec, ticks, part, part_end, parts)
    t, err = CudaTune(), _err()
    L = lib()
    L.cuda_enum_tune.restype = C.c_int
    L.cuda_enum_tune.argtypes = [C.POINTER(EnumStruct), C.POINTER(CudaTune), C.c_char_p,
                                 C.c_size_t]
    if not L.cuda_enum_tune(C.byref(e), C.byref(t), err, len(err)):
        raise EngineError(err.value.decode())
    cands = [{"block": t.cand[i].block, "step_bits": t.cand[i].step_bits,
              "ms": t.cand[i].ms if t.cand[i].ms >= 0 else None} for i in range(t.n)]
    return {"candidates": cands, "best": cands[t.best], "probe_fraction": t.probe_fraction}


def table(p: Program, ticks: int = 1):
    """`run --table --engine cuda` (cuda_table): every row's output columns (.out cells, or RR
    when there are none) as a list of rows of 0/1."""
    rows, cols = 1 << p.s.ninputs, max(p.s.noutputs, 1)
    vals = (C.c_uint8 * (rows * cols))() if 0 < p.s.ninputs <= 20 else (C.c_uint8 * 1)()
    err = _err()
    L = lib()
    L.cuda_table.restype = C.c_int
    L.cuda_table.argtypes = [C.POINTER(ProgramStruct), C.c_uint, C.c_void_p, C.c_char_p,
                             C.c_size_t]
    if not L.cuda_table(p.ptr, ticks, C.cast(vals, C.c_void_p), err, len(err)):
        raise EngineError(err.value.decode())
    return [list(vals[r * cols:(r + 1) * cols]) for r in range(rows)]


def last_launch() -> dict:
    s = LaunchStats()
    lib().cuda_last_launch(C.byref(s))
    return {f: getattr(s, f) for f, _ in LaunchStats._fields_}


def lop3_peak() -> float:
    """Measured 32-bit LOP3 operations per second of the device (the roofline denominator)."""
    ops, sec, err = C.c_double(), C.c_double(), _err()
    if not lib().cuda_lop3_peak(C.byref(ops), C.byref(sec), err, len(err)):
        raise EngineError(err.value.decode())
    return ops.value


def batch_run(jobs) -> list:
    """Many enumerations in one persistent launch (cuda_batch_run).  jobs: iterable of dicts
    with keys mode, a, b, spec, ticks.  Returns one result dict per job."""
    jobs = list(jobs)
    n = len(jobs)
    structs = [make_enum(j["mode"], j["a"], j.get("b"), j.get("spec"), j.get("ticks", 1))
               for j in jobs]
    arr = (C.POINTER(EnumStruct) * max(n, 1))(*[C.pointer(s) for s in structs])
    res = (EnumResult * max(n, 1))()
    err = _err()
    L = lib()
    L.cuda_batch_run.restype = C.c_int
    L.cuda_batch_run.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_char_p, C.c_size_t]
    if not L.cuda_batch_run(C.cast(arr, C.c_void_p), n, C.cast(res, C.c_void_p), err, len(err)):
        raise EngineError(err.value.decode())
    return [res[i].as_dict() for i in range(n)]


def batch_prepare(jobs) -> int:
    """Compiles and loads the quick-start kernel of every job a batch_run of these jobs could run
    as generated code (cuda_batch_prepare); returns how many."""
    jobs = list(jobs)
    n = len(jobs)
    structs = [make_enum(j["mode"], j["a"], j.get("b"), j.get("spec"), j.get("ticks", 1))
               for j in jobs]
    arr = (C.POINTER(EnumStruct) * max(n, 1))(*[C.pointer(s) for s in structs])
    got, err = C.c_int(), _err()
    L = lib()
    L.cuda_batch_prepare.restype = C.c_int
    L.cuda_batch_prepare.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_int), C.c_char_p,
                                     C.c_size_t]
    if not L.cuda_batch_prepare(C.cast(arr, C.c_void_p), n, C.byref(got), err, len(err)):
        raise EngineError(err.value.decode())
    return got.value


class BatchStats(C.Structure):
    _fields_ = [("jobs", C.c_int), ("compiled", C.c_int), ("interpreted", C.c_int),
                ("compile_threads", C.c_int), ("planned", C.c_int), ("taken_back", C.c_int),
                ("seconds", C.c_double), ("interpreter_start", C.c_double),
                ("interpreter_end", C.c_double), ("compiled_end", C.c_double),
                ("compile_busy", C.c_double), ("compile_load", C.c_double),
                ("loop_end", C.c_double)]


def batch_stats() -> dict:
    """The last batch_run: jobs on generated kernels and on the interpreter, compile threads,
    wall seconds (cuda_batch_stats)."""
    s = BatchStats()
    lib().cuda_batch_stats(C.byref(s))
    return {f: getattr(s, f) for f, _ in BatchStats._fields_}


SERVE_AUTO, SERVE_INTERPRETER, SERVE_COMPILED = 0, 1, 2


class ServeOpts(C.Structure):
    _fields_ = [("streams", C.c_int), ("max_inflight_jobs", C.c_int),
                ("max_device_bytes", C.c_size_t), ("max_wave_jobs", C.c_int),
                ("share", C.c_double), ("compile_threads", C.c_int),
                ("compiled_slots", C.c_int), ("route", C.c_int)]


def serve_run(jobs, arrivals, streams=4, max_inflight_jobs=0, max_device_bytes=0,
              max_wave_jobs=0, share=0.0, compile_threads=0, compiled_slots=0,
              route=SERVE_AUTO, engines=None):
    """Continuous-batching serving (cuda_serve_run): job i arrives arrivals[i] seconds after
    the call starts.  Returns (results, start, finish), times in seconds from the start; a list
    passed as `engines` gets each job's engine (0 interpreter, 1 generated code)."""
    jobs = list(jobs)
    n = len(jobs)
    structs = [make_enum(j["mode"], j["a"], j.get("b"), j.get("spec"), j.get("ticks", 1))
               for j in jobs]
    arr = (C.POINTER(EnumStruct) * max(n, 1))(*[C.pointer(x) for x in structs])
    at = (C.c_double * max(n, 1))(*arrivals)
    start = (C.c_double * max(n, 1))()
    finish = (C.c_double * max(n, 1))()
    res = (EnumResult * max(n, 1))()
    used = (C.c_int * max(n, 1))()
    o = ServeOpts(streams, max_inflight_jobs, max_device_bytes, max_wave_jobs, share,
                  compile_threads, compiled_slots, route)
    err = _err()
    L = lib()
    L.cuda_serve_run.restype = C.c_int
    L.cuda_serve_run.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.POINTER(ServeOpts),
                                 C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_char_p,
                                 C.c_size_t]
    if not L.cuda_serve_run(C.cast(arr, C.c_void_p), C.cast(at, C.c_void_p), n, C.byref(o),
                            C.cast(start, C.c_void_p), C.cast(finish, C.c_void_p),
                            C.cast(res, C.c_void_p), C.cast(used, C.c_void_p), err, len(err)):
        raise EngineError(err.value.decode())
    if engines is not None:
        engines[:] = list(used[:n])
    return [res[i].as_dict() for i in range(n)], list(start[:n]), list(finish[:n])


def super_parse(text: str) -> SuperSpec:
    sp, err = SuperSpec(), _err()
    L = lib()
    L.cuda_super_parse.restype = C.c_int
    L.cuda_super_parse.argtypes = [C.c_char_p, C.POINTER(SuperSpec), C.c_char_p, C.c_size_t]
    if not L.cuda_super_parse(text.encode(), C.byref(sp), err, len(err)):
        raise EngineError(err.value.decode())
    return sp


def super_search(text: str, max_cost: int = 30, quiet: bool = True) -> dict:
    """`alpha super SPEC` on the GPU: the shortest NAND/STO program, proven (cuda_super_search)."""
    sp = super_parse(text)
    o = SuperOpts(0, 0, 1, max_cost, int(quiet))
    r, err = SuperResult(), _err()
    L = lib()
    L.cuda_super_search.restype = C.c_int
    L.cuda_super_search.argtypes = [C.POINTER(SuperSpec), C.POINTER(SuperOpts),
                                    C.POINTER(SuperResult), C.c_char_p, C.c_size_t]
    if not L.cuda_super_search(C.byref(sp), C.byref(o), C.byref(r), err, len(err)):
        raise EngineError(err.value.decode())
    prog = [("NAND" if r.prog.code[i].op == OP_NAND else "STO", r.prog.code[i].cell.decode())
            for i in range(r.prog.len)] if r.found else []
    ok, why = super_check(sp, r.prog) if r.found else (False, "")
    return {"found": bool(r.found), "cost": r.cost, "below": r.below,
            "contradiction": bool(r.contradiction), "nodes": r.nodes, "seconds": r.seconds,
            "program": prog, "checked": ok, "check_error": why}


def super_check(sp: SuperSpec, prog: SuperProg):
    err = _err()
    L = lib()
    L.cuda_super_check.restype = C.c_int
    L.cuda_super_check.argtypes = [C.POINTER(SuperSpec), C.POINTER(SuperProg), C.c_char_p,
                                   C.c_size_t]
    ok = L.cuda_super_check(C.byref(sp), C.byref(prog), err, len(err))
    return bool(ok), err.value.decode()


def check(program: Program, seed: int = 1, ticks: int = 8) -> dict:
    """`alpha check --engine cuda` (check_lanes, src/check.c:52-113): random state, `ticks`
    passes on the GPU, every machine compared with the reference machine after every tick."""
    r, err = CheckResult(), _err()
    if not lib().cuda_check(program.ptr, seed, ticks, C.byref(r), err, len(err)):
        raise EngineError(err.value.decode())
    return {f: getattr(r, f) for f, _ in CheckResult._fields_}


class DemoResult(C.Structure):
    _fields_ = [("what", C.c_char * 96), ("instr", C.c_size_t), ("segs", C.c_uint),
                ("kernels", C.c_uint), ("ok", C.c_int), ("pass_seconds", C.c_double),
                ("passes_per_second", C.c_double)]


def cube_demo(name: str, dims: int, checks: int = 3, seconds: float = 0.2) -> dict:
    """`alpha cube DEMO --dims D` (cuda_cube_demo): checked rounds, then passes per second."""
    r, e = DemoResult(), _err()
    L = lib()
    L.cuda_cube_demo.restype = C.c_int
    L.cuda_cube_demo.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_double,
                                 C.POINTER(DemoResult), C.c_char_p, C.c_size_t]
    if not L.cuda_cube_demo(name.encode(), dims, checks, seconds, C.byref(r), e, len(e)):
        raise EngineError(e.value.decode())
    return {f: (getattr(r, f).decode() if f == "what" else getattr(r, f))
            for f, _ in DemoResult._fields_}


class _CubeCand(C.Structure):
    _fields_ = [("warps", C.c_uint), ("iters", C.c_uint), ("ms", C.c_double)]


class CudaCubeTune(C.Structure):
    _fields_ = [("n", C.c_int), ("best", C.c_int), ("cand", _CubeCand * 8),
                ("probe_passes", C.c_uint)]


class Cube:
    """A program's cube of machines on the device (LaneCube + jit_cube_run).

    words are cell-major: cell c of machine m is bit m % 32 of word c * W + m // 32, W = machines
    // 32; RR is W more words.  load/store move one group of 512 machines in the reference's
    Line layout: ncells lines of 8 uint64."""

    def __init__(self, program: Program):
        import numpy as np
        self.np = np
        self.program = program
        self.h = C.c_void_p()
        e = _err()
        if not lib().cuda_cube_new(program.ptr, C.byref(self.h), e, len(e)):
            raise EngineError(e.value.decode())
        self.groups = lib().cuda_cube_groups(self.h)
        self.machines = self.groups * 512
        self.W = self.machines // 32
        self.segments = lib().cuda_cube_segments(self.h)
        self.kernels = lib().cuda_cube_kernels(self.h)
        self.closing_copies = lib().cuda_cube_closing_copies(self.h)

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.cuda_cube_free(self.h)
            self.h = None

    def run(self, passes: int = 1) -> float:
        e = _err()
        if not lib().cuda_cube_run(self.h, passes, e, len(e)):
            raise EngineError(e.value.decode())
        return last_launch()["kernel_ms"]

    def tune(self, probe_passes: int = 16) -> dict:
        """The cube's autotuner (cuda_cube_tune): warps and word runs per group-major block,
        measured on this cube from its present state, which it leaves unchanged."""
        t, e = CudaCubeTune(), _err()
        L = lib()
        L.cuda_cube_tune.restype = C.c_int
        L.cuda_cube_tune.argtypes = [C.c_void_p, C.c_uint, C.POINTER(CudaCubeTune), C.c_char_p,
                                     C.c_size_t]
        if not L.cuda_cube_tune(self.h, probe_passes, C.byref(t), e, len(e)):
            raise EngineError(e.value.decode())
        cands = [{"warps": t.cand[i].warps, "iters": t.cand[i].iters,
                  "ms": t.cand[i].ms if t.cand[i].ms >= 0 else None} for i in range(t.n)]
        return {"candidates": cands, "best": cands[t.best], "probe_passes": probe_passes}

    def read(self):
        np = self.np
        mem = np.zeros(self.program.ncells * self.W, dtype=np.uint32)
        rr = np.zeros(self.W, dtype=np.uint32)
        e = _err()
        if not lib().cuda_cube_read_words(self.h, mem.ctypes.data, rr.ctypes.data, e, len(e)):
            raise EngineError(e.value.decode())
        return mem.reshape(self.program.ncells, self.W), rr

    def write(self, mem, rr=None):
        np = self.np
        mem = np.ascontiguousarray(mem, dtype=np.uint32)
        rr = None if rr is None else np.ascontiguousarray(rr, dtype=np.uint32)
        e = _err()
        if not lib().cuda_cube_write_words(self.h, mem.ctypes.data,
                                           None if rr is None else rr.ctypes.data, e, len(e)):
            raise EngineError(e.value.decode())

    def load_group(self, g, lines, rr_line=None):
        np = self.np
        lines = np.ascontiguousarray(lines, dtype=np.uint64)
        rr_line = None if rr_line is None else np.ascontiguousarray(rr_line, dtype=np.uint64)
        e = _err()
        if not lib().cuda_cube_load(self.h, g, lines.ctypes.data,
                                    None if rr_line is None else rr_line.ctypes.data, e, len(e)):
            raise EngineError(e.value.decode())

    def store_group(self, g):
        np = self.np
        lines = np.zeros((self.program.ncells, 8), dtype=np.uint64)
        rr = np.zeros(8, dtype=np.uint64)
        e = _err()
        if not lib().cuda_cube_store(self.h, g, lines.ctypes.data, rr.ctypes.data, e, len(e)):
            raise EngineError(e.value.decode())
        return lines, rr


def device_info() -> str:
    buf = C.create_string_buffer(512)
    if not lib().cuda_device_info(buf, len(buf)):
        raise EngineError(buf.value.decode())
    return buf.value.decode()


def codegen_enum_source(mode, a: Program, b: Program | None = None, spec: Spec | None = None,
                        ticks=1) -> str:
    """The CUDA C the engine generates for an enumeration (for inspection and host tests)."""
    return _codegen(mode, a, b, spec, ticks)


def codegen_ptx_source(mode, a: Program, b: Program | None = None, spec: Spec | None = None,
                       target: str = "sm_103a") -> str:
    """The PTX the engine writes directly for a quick-start build of an equivalence or search job
    (ptxgen.c), for the .target given (for inspection and ptxas tests)."""
    return codegen_ptx_module([(mode, a, b, spec)], target)


def codegen_ptx_module(jobs, target: str = "sm_103a") -> str:
    """The PTX module of several (mode, a, b, spec) jobs built together: kernels tc_enum_0 .. ."""
    L = lib()
    fn = L.tc_codegen_ptx_for
    fn.restype = C.c_void_p
    fn.argtypes = [C.POINTER(C.POINTER(EnumStruct)), C.c_int, C.c_char_p,
                   C.POINTER(C.c_size_t), C.c_char_p, C.c_size_t]
    es = [make_enum(*j) for j in jobs]
    arr = (C.POINTER(EnumStruct) * len(es))(*[C.pointer(e) for e in es])
    n, err = C.c_size_t(), _err()
    p = fn(arr, len(es), target.encode(), C.byref(n), err, len(err))
    if not p:
        raise EngineError(err.value.decode())
    s = C.string_at(p, n.value).decode()
    L.tc_free.argtypes = [C.c_void_p]
    L.tc_free(p)
    return s


def set_enum_ptx(on: bool) -> bool:
    """Switches the quick-start builds of equivalence and search jobs between PTX written directly
    (on, the default) and CUDA C through NVRTC; returns the previous setting."""
    v = C.c_int.in_dll(lib(), "tc_enum_ptx")
    old = bool(v.value)
    v.value = 1 if on else 0
    return old


def set_enum_quick(on: bool) -> bool:
    """Makes enum_run build and run quick-start kernels, as a batch's compiled jobs are built (PTX
    written directly for equivalence and search jobs), even where the optimised kernel of the same
    job is cached; returns the previous setting."""
    v = C.c_int.in_dll(lib(), "tc_enum_run_fast")
    old = bool(v.value)
    v.value = 2 if on else 0
    return old


def _codegen(mode, a, b, spec, ticks):
    L = lib()
    fn = L.tc_codegen_enum_for
    fn.restype = C.c_void_p
    fn.argtypes = [C.POINTER(EnumStruct), C.POINTER(C.c_size_t), C.c_char_p, C.c_size_t]
    e = make_enum(mode, a, b, spec, ticks)
    n, err = C.c_size_t(), _err()
    p = fn(C.byref(e), C.byref(n), err, len(err))
    if not p:
        raise EngineError(err.value.decode())
    s = C.string_at(p, n.value).decode()
    L.tc_free.argtypes = [C.c_void_p]
    L.tc_free(p)
    return s
