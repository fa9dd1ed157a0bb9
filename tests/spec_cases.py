"""Seeded specification texts for the parser's parity tests: well-formed expressions over the
operators and vectors of a few program headers, and the same texts damaged (characters deleted,
inserted, doubled), nested past the evaluation stack, or longer than the RPN holds.

Used by tests/test_spec_parity.py (against the reference's spec_parse where it is built here,
else against tests/golden/spec.json) and by tests/golden/make_spec_golden.py, which wrote that
fixture from the reference."""
from __future__ import annotations

import random

# Program headers: the reference's 8-bit adder (tests/test_work.c:190-205), and one whose names
# exercise vector resolution: an exact name that is also a stem (y, y3), a gap (w0 w2), a leading
# zero (q00), a bit index of 64 (v64), mixed case (Z0 z1), a 40-bit vector.
HEADERS = {
    "adder": (".in  a7 a6 a5 a4 a3 a2 a1 a0  b7 b6 b5 b4 b3 b2 b1 b0  c\n"
              ".out s7 s6 s5 s4 s3 s2 s1 s0  c\n"),
    "names": (".in x0 x1 x2 y y3 Z0 z1 q00 q1 w0 w2 v0 v64 " +
              " ".join(f"m{i}" for i in range(40)) + "\n"
              ".out o0 o1 o2 o3 r R1 t0 t2 k Kk " + " ".join(f"e{i}" for i in range(60)) + "\n"),
}
# (good inputs, bad inputs, good left sides, bad left sides)
NAMES = {
    "adder": (["a", "b", "c", "A", "B"], ["a3", "s", "zz"],
              ["s", "c", "S", "s:c", "c:s", "c : s"], ["q", "s:", ":s"]),
    "names": (["x", "X", "y", "y3", "Z", "z", "q00", "m", "M", "x1"], ["q", "w", "v", "nope"],
              ["o", "r", "R", "k", "Kk", "e", "o:r", "e:o", "r:k:o", "e:r:k:Kk"],
              ["t", "e:e", "t:o", "o:e:o"]),
}
BINARY = ["+", "-", "*", "&", "|", "^", "<<", ">>"]
JUNK = "()~-+*<>&^|=:xyzab0123 \t\n_.#"


def number(rng: random.Random) -> str:
    v = rng.choice([0, 1, 2, 3, 7, 8, 15, 63, 64, 65, 255, 0xffff, 2**63, 2**64 - 1,
                    rng.getrandbits(rng.choice([4, 16, 40, 64]))])
    form = rng.random()
    if form < 0.5:
        return str(v)
    if form < 0.8:
        return hex(v) if rng.random() < 0.5 else "0X%X" % v
    return "0" + oct(v)[2:] if v else "0"


def expression(rng: random.Random, names, depth: int) -> str:
    r = rng.random()
    if depth <= 0 or r < 0.25:
        return rng.choice(names) if rng.random() < 0.6 else number(rng)
    if r < 0.4:
        return rng.choice(["~", "-", "- ", "~ ~"]) + expression(rng, names, depth - 1)
    if r < 0.55:
        return "(" + rng.choice(["", " "]) + expression(rng, names, depth - 1) + ")"
    sp = rng.choice(["", " ", "\t", "  "])
    return (expression(rng, names, depth - 1) + sp + rng.choice(BINARY) + sp +
            expression(rng, names, depth - 1))


def damage(rng: random.Random, text: str) -> str:
    for _ in range(rng.randint(1, 3)):
        i = rng.randrange(len(text) + 1)
        k = rng.random()
        if k < 0.4 and text:
            text = text[:i] + text[i + 1:]
        elif k < 0.8:
            text = text[:i] + rng.choice(JUNK) + text[i:]
        else:
            j = min(len(text), i + rng.randint(1, 4))
            text = text[:j] + text[i:j] + text[j:]
    return text


def cases(n: int, seed: int = 2024):
    """(header, text, inputs_allowed) triples, deterministic in n and seed."""
    rng = random.Random(seed)
    out = []
    for i in range(n):
        h = rng.choice(sorted(HEADERS))
        good_in, bad_in, good_out, bad_out = NAMES[h]
        ins = good_in + (bad_in if rng.random() < 0.15 else [])
        lhs = rng.choice(bad_out if rng.random() < 0.08 else good_out)
        rhs = expression(rng, ins, rng.randint(0, 7))
        text = lhs + rng.choice([" = ", "=", " =\t", " = "]) + rhs
        k = rng.random()
        if k < 0.3:
            text = damage(rng, text)
        elif k < 0.36:
            d = rng.choice([62, 63, 64, 65, 70])   # parentheses nest operands on the stack
            text = lhs + " = " + "".join(f"{rng.choice(ins)} {rng.choice(BINARY)} ("
                                         for _ in range(d)) + "1" + ")" * d
            if rng.random() < 0.5:
                text = damage(rng, text)
        elif k < 0.42:
            m = rng.choice([120, 127, 128, 129, 200])  # 2m - 1 RPN items
            text = lhs + " = " + " + ".join(rng.choice(ins + ["1"]) for _ in range(m))
            if rng.random() < 0.5:
                text = text + rng.choice([" )", " x", " +", ""])
        elif k < 0.45:
            text = lhs + " = " + "-" * rng.randint(250, 260) + rng.choice(ins)
        out.append((h, text, rng.random() < 0.85))
    return out
