"""Seeded assembly sources for the assembler's parity tests.

Each case is a source text plus a set of include files: declarations (.in/.out, with id cells,
constants and repeats), NAND/STO lines, links (with blanks, odd dimensions, loops, late
declarations), macros (parameters, '#' joins, @locals, numbers and locals as arguments, calls of
other macros, recursion, wrong argument counts, macros defined in included files), quoted
tokens, commas and comments, and the same sources damaged (characters deleted, inserted,
doubled).  Includes are named relative to the source's directory, so a run needs only the
files written next to it (write_includes) and the base directory ".".

Used by tests/test_asm_parity.py (against the reference's asm_string where it is built here,
else against tests/golden/asm.json) and by tests/golden/make_asm_golden.py, which wrote that
fixture from the reference."""
from __future__ import annotations

import ctypes as C
import hashlib
import os
import random

INCLUDES = {
    "std.inc": (".macro NOT a\nNAND a\n.endm\n"
                ".macro LD a\nNAND ONE\nNAND a\nNAND ONE\n.endm\n"
                ".macro MOV d s\nLD s\nSTO d\n.endm\n"
                ".macro XOR r x y\nLD x\nNAND y\nSTO @t\nNAND x\nSTO @u\nLD @t\nNAND y\n"
                "NAND @u\nSTO r\n.endm\n"),
    "bits.inc": (".macro SET2 v\nNAND ZERO\nSTO v#0\nSTO v#1\n.endm\n"
                 ".macro PICK v d\nNAND v#d\nNAND ID#d\n.endm\n"),
    "nested.inc": ".include \"std.inc\"\n.in n0 n1\nMOV n1 n0\n",
    "bad.inc": "NAND a\nSTO ONE\n",
    "local.inc": "STO @inside\n",
    "sub/deep.inc": ".include \"../bits.inc\"\nNAND deep\n",
}
NAMES = ["a", "b", "c", "x", "y", "sum0", "sum1", "Sum2", "ID0", "ID3", "id9", "ID15", "ID16",
         "ID01", "ZERO", "ONE", "one", "t_1", "_u", "A", "B"]
BAD_NAMES = ["1x", "@t", "a-b", "\"a b\"", "\"\"", "x.y", "@", "#"]


def write_includes(directory: str) -> None:
    for name, text in INCLUDES.items():
        path = os.path.join(directory, name)
        os.makedirs(os.path.dirname(path), exist_ok=True)
        with open(path, "w") as f:
            f.write(text)


def _name(rng, bad=0.04):
    return rng.choice(BAD_NAMES) if rng.random() < bad else rng.choice(NAMES)


def _sep(rng):
    return rng.choice([" ", "  ", "\t", ", ", ",", " , "])


def _macro(rng, name, nparams, callables):
    params = ["p", "q", "r", "v", "d"][:nparams]
    body = []
    for _ in range(rng.randint(0, 5)):
        k = rng.random()
        pool = params + ["@t", "@u", "w", "ONE"]
        if k < 0.35:
            body.append(f"    NAND {rng.choice(pool)}")
        elif k < 0.6:
            body.append(f"    STO {rng.choice([p for p in pool if p != 'ONE'] or ['w'])}")
        elif k < 0.7 and params:
            body.append(f"    NAND {rng.choice(params)}#{rng.choice(['0', '1'] + params)}")
        elif k < 0.75:
            body.append(f"    NAND ID#{rng.choice(params + ['2'])}")
        elif k < 0.9 and callables:
            m, n = rng.choice(callables)
            body.append("    " + m + "".join(" " + rng.choice(pool + ["7"]) for _ in range(n)))
        else:
            body.append("    ; a comment")
    head = ".macro " + name + "".join(" " + p for p in params)
    return [head] + body + [".endm"]


def source(rng) -> str:
    lines = []
    macros = []
    if rng.random() < 0.4:
        lines.append('.include "' + rng.choice(sorted(INCLUDES) + ["missing.inc"]) + '"')
        if "std.inc" in lines[-1]:
            macros += [("NOT", 1), ("LD", 1), ("MOV", 2), ("XOR", 3)]
        if "bits.inc" in lines[-1] or "deep.inc" in lines[-1]:
            macros += [("SET2", 1), ("PICK", 2)]
    for _ in range(rng.randint(1, 14)):
        k = rng.random()
        if k < 0.12:
            lines.append(rng.choice([".in", ".out", ".IN", ".Out"]) +
                         "".join(_sep(rng) + _name(rng) for _ in range(rng.randint(0, 4))))
        elif k < 0.45:
            op = rng.choice(["NAND", "STO", "nand", "Sto"])
            args = [_name(rng) for _ in range(1 if rng.random() < 0.93 else rng.choice([0, 2]))]
            lines.append("    " + op + "".join(_sep(rng) + a for a in args) +
                         rng.choice(["", "", " ; note", ";x"]))
        elif k < 0.55:
            y, x = rng.choice(["ly", "lz", "a", "ID2", "lw"]), _name(rng)
            d = rng.choice(["0", "3", "8", "9", "15", "16", "-1", "", "x", "+2", "03"])
            sp = rng.choice(["", " "])
            lines.append(f".link {y}{sp}={sp}{x}{sp}@{sp}{d}" if rng.random() < 0.9
                         else f".link {y} {x} {d}")
        elif k < 0.7:
            name = rng.choice(["M", "N", "K", "m", "NAND", "1M", "XOR"])
            if any(n == name.upper() for n, _ in macros) and rng.random() < 0.8:
                continue
            nparams = rng.randint(0, 3)
            lines += _macro(rng, name, nparams, macros)
            if rng.random() < 0.05:
                lines.pop()  # no .endm
            macros.append((name.upper(), nparams))
        elif k < 0.9 and macros:
            m, n = rng.choice(macros)
            n = n if rng.random() < 0.92 else n + rng.choice([-1, 1])
            args = [rng.choice(NAMES + ["5", "12", "\"sp ace\""] + BAD_NAMES[:1])
                    for _ in range(max(n, 0))]
            lines.append("  " + rng.choice([m, m.lower()]) + "".join(_sep(rng) + a for a in args))
        elif k < 0.95:
            lines.append(rng.choice(["", "   ", "; only a comment", ".endm", ".bogus x",
                                     '.include', '.include "std.inc" "x"', "\t\r", '"unterminated',
                                     "NAND \"q r\"", "STO a, , ,"]))
        else:
            lines.append('.include "' + rng.choice(["bad.inc", "local.inc", "nested.inc",
                                                    "sub/deep.inc", "nope/x.inc"]) + '"')
    text = "\n".join(lines) + rng.choice(["\n", "", "\n\n"])
    if rng.random() < 0.15:
        for _ in range(rng.randint(1, 3)):
            i = rng.randrange(len(text) + 1)
            r = rng.random()
            if r < 0.4 and text:
                text = text[:i] + text[i + 1:]
            elif r < 0.8:
                text = text[:i] + rng.choice("\n ;,\"@#.=") + text[i:]
            else:
                j = min(len(text), i + rng.randint(1, 6))
                text = text[:j] + text[i:j] + text[j:]
    return text


WRITABLE = ["a", "b", "c", "x", "y", "sum0", "sum1", "Sum2", "t_1", "_u", "A", "B", "ID01"]
READABLE = WRITABLE + ["ID0", "ID3", "id9", "ID15", "ZERO", "ONE", "one"]


def clean_source(rng) -> str:
    """A source that assembles: every name valid, stores only to writable cells, links declared
    before use with dimensions 0..15, macros defined once and called with their arity."""
    lines, macros, links = [], [], 0
    if rng.random() < 0.5:
        inc = rng.choice(["std.inc", "bits.inc", "nested.inc", "sub/deep.inc"])
        lines.append(f'.include "{inc}"')
        if inc in ("std.inc", "nested.inc"):
            macros += [("NOT", ["a"]), ("LD", ["a"]), ("MOV", ["w", "r"]), ("XOR", ["w", "r", "r"])]
        else:
            macros += [("SET2", ["v"]), ("PICK", ["v", "d"])]
    declared = set()
    for _ in range(rng.randint(2, 20)):
        k = rng.random()
        if k < 0.12:
            which = rng.choice([".in", ".out"])
            fresh = sorted({n.lower() for n in WRITABLE} - {d for w, d in declared if w == which})
            pick = rng.sample(fresh, min(len(fresh), rng.randint(1, 3)))
            if pick:
                lines.append(which + "".join(_sep(rng) + n for n in pick))
                declared |= {(which, n) for n in pick}
        elif k < 0.55:
            if rng.random() < 0.5:
                lines.append("    NAND " + rng.choice(READABLE + [f"l{i}" for i in range(links)]))
            else:
                lines.append("    STO " + rng.choice(WRITABLE))
        elif k < 0.65:
            src = rng.choice(READABLE + [f"l{i}" for i in range(links)])
            d = rng.randint(0, 15)
            sp = rng.choice(["", " ", "\t"])
            lines.append(f".link l{links}{sp}={sp}{src}{sp}@{sp}{d}")
            links += 1
        elif k < 0.78:
            name = f"M{len(macros)}"
            params = ["p", "q", "v"][:rng.randint(0, 3)]
            body = []
            for _ in range(rng.randint(1, 6)):
                r = rng.random()
                if r < 0.3:
                    body.append("  NAND " + rng.choice(params + ["@t", "@u", "ONE", "ID2"]))
                elif r < 0.55:
                    body.append("  STO " + rng.choice(params + ["@t", "@u", "w"]))
                elif r < 0.7 and "v" in params:
                    body.append("  NAND v#" + rng.choice(["0", "1", "2"]))
                elif r < 0.9 and macros:
                    m, ps = rng.choice(macros)
                    body.append("  " + m + "".join(
                        " " + rng.choice(params + ["@t", "@u", "w"]) if p != "d" else " 3"
                        for p in ps))
                else:
                    body.append("  ; comment")
            lines += [f".macro {name} " + " ".join(params)] + body + [".endm"]
            macros.append((name, params))
        elif macros:
            m, ps = rng.choice(macros)
            lines.append("  " + m.lower() + "".join(
                _sep(rng) + (rng.choice(WRITABLE) if p != "d" else str(rng.randint(0, 15)))
                for p in ps))
    return "\n".join(lines) + "\n"


def cases(n: int, seed: int = 99):
    rng = random.Random(seed)
    return [clean_source(rng) if rng.random() < 0.7 else source(rng) for _ in range(n)]


def digest(p) -> str:
    """sha256 (first 24 hex digits) of a ProgramStruct's contents: code, names, inputs,
    outputs and, when present, the per-cell kinds."""
    h = hashlib.sha256()
    h.update(b"%d %d %d %d|" % (p.len, p.ncells, p.ninputs, p.noutputs))
    h.update(b"".join(b"%d.%d," % (p.code[i].op, p.code[i].addr) for i in range(p.len)))
    for i in range(p.ncells):
        h.update(p.cell_names[i] + b"\0")
    h.update(bytes(C.string_at(p.inputs, 4 * p.ninputs)) if p.ninputs else b"")
    h.update(bytes(C.string_at(p.outputs, 4 * p.noutputs)) if p.noutputs else b"")
    if p.special:
        for i in range(p.ncells):
            s = p.special[i]
            h.update(b"%d:%d:%d," % (s.kind, s.dim, s.src))
    return h.hexdigest()[:24]
