"""Seeded superoptimizer specifications and programs for the parity tests of the spec parser
and the program check.

Texts: one to five statements over a few names, RR and constants with ! ~ & ^ | ?: and
parentheses, outputs with {input} sharing, given cells (:=), statements repeated or contradicting
(set twice, RR given, sharing with an output), too many inputs, names of 23 characters and more,
and damaged texts.  Programs: random NAND/STO sequences over ZERO, ONE, the spec's cells and
scratch cells, for valid specs.

Used by tests/test_super_parity.py (against the reference where it is built here, else against
tests/golden/super.json) and by tests/golden/make_super_golden.py, which wrote that fixture."""
from __future__ import annotations

import random

NAMES = ["a", "b", "c", "x", "y", "s", "n", "RR", "rr", "g", "d", "e", "f",
         "averyveryverylongname_0123", "h"]


def expr(rng, names, depth):
    r = rng.random()
    if depth <= 0 or r < 0.3:
        return rng.choice(names + ["0", "1"]) if rng.random() < 0.9 else rng.choice(names)
    if r < 0.42:
        return rng.choice(["!", "~", "! "]) + expr(rng, names, depth - 1)
    if r < 0.52:
        return "(" + expr(rng, names, depth - 1) + ")"
    if r < 0.6:
        return (expr(rng, names, depth - 1) + " ? " + expr(rng, names, depth - 1) + " : " +
                expr(rng, names, depth - 1))
    sp = rng.choice(["", " ", "\n"])
    return expr(rng, names, depth - 1) + sp + rng.choice("&^|") + sp + expr(rng, names, depth - 1)


def spec_text(rng) -> str:
    k = rng.randint(1, 4)
    names = rng.sample(NAMES[:12], rng.randint(2, 7)) + \
        (["averyveryverylongname_0123"] if rng.random() < 0.03 else [])
    stmts = []
    for _ in range(k):
        lhs = rng.choice(names + ["RR", "o", "p", "q"])
        alias = ""
        if rng.random() < 0.25:
            alias = "{" + ",".join(rng.sample(names, rng.randint(1, min(3, len(names))))) + "}"
        op = " := " if rng.random() < 0.12 else rng.choice([" = ", "=", " =\t"])
        stmts.append(lhs + alias + op + expr(rng, names, rng.randint(0, 4)))
    text = rng.choice(["; ", ";", " ;\n"]).join(stmts) + rng.choice(["", ";", " ", "; "])
    if rng.random() < 0.2:
        for _ in range(rng.randint(1, 2)):
            i = rng.randrange(len(text) + 1)
            if rng.random() < 0.5 and text:
                text = text[:i] + text[i + 1:]
            else:
                text = text[:i] + rng.choice("(){},;:=?!&^|01ab ") + text[i:]
    return text


def spec_texts(n: int, seed: int = 5):
    rng = random.Random(seed)
    return [spec_text(rng) for _ in range(n)]


# Specifications whose shortest programs the reference's own search finds in well under a second
# (its tests/test_super.c:159-172 list and a few more with sharing, given cells and RR).
SEARCHED = ["RR = 1", "RR = !RR", "RR = 0", "RR = x", "RR = !x", "RR = RR & x", "RR = RR | x",
            "RR = !(RR | x)", "RR = RR & !x", "RR = RR | !x", "x = !RR; RR = RR",
            "dst = src; RR = src", "r = r | n", "r = r & n", "m = id & n", "o{x,y} = x & y",
            "o{x,y} = x | y", "RR = RR ^ x", "RR = !(RR ^ x)", "r = r ^ n", "o{x,y} = x ^ y",
            "r{a,b} = s ? a : b", "o{a0,a1} = s ? a1 : a0; ns := !s", "p = a & b; q = a | b",
            "RR = a ^ b; c = a & b", "o{a,b} = a & !b | !a & b", "t = !t; RR = t",
            "u = a ? b : 0; v = a ? 0 : b"]


def mutants(rng, code, cells, n):
    """n programs one edit away from code: an instruction's cell or opcode changed, one
    deleted, one inserted, or two exchanged."""
    pool = ["ZERO", "ONE"] + cells + ["_t1", "_t2", "_t3"]
    out = []
    for _ in range(n):
        c = list(code)
        k = rng.random()
        i = rng.randrange(len(c)) if c else 0
        if k < 0.35 and c:
            c[i] = (c[i][0], rng.choice(pool[2:] if c[i][0] else pool))
        elif k < 0.5 and c and c[i][1] not in ("ZERO", "ONE"):
            c[i] = (1 - c[i][0], c[i][1])
        elif k < 0.65 and c:
            del c[i]
        elif k < 0.85 and len(c) < 60:
            op = int(rng.random() < 0.4)
            c.insert(rng.randrange(len(c) + 1), (op, rng.choice(pool[2:] if op else pool)))
        elif len(c) > 1:
            j = rng.randrange(len(c))
            c[i], c[j] = c[j], c[i]
        out.append(c)
    return out


def program(rng, cells, maxlen=24):
    """A random program as (op, cell) pairs: 0 NAND, 1 STO."""
    pool = ["ZERO", "ONE"] + cells + ["_t1", "_t2", "_t3"]
    code = []
    for _ in range(rng.randint(0, maxlen)):
        op = rng.random() < 0.4
        cell = rng.choice(pool[2:] if op and rng.random() < 0.97 else pool)
        code.append((int(op), cell))
    return code
