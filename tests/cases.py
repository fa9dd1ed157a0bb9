"""Shared helpers: golden cases and programs built by the engine's own generators."""
from __future__ import annotations

import json
import os

import tesseract_gb300 as T

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
MODES = {"verify": T.EN_VERIFY, "equiv": T.EN_EQUIV, "search": T.EN_SEARCH}


def load(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


def program(desc):
    kind, p = desc["kind"], desc["params"]
    if kind == "mul":
        return T.Program.gen_mul(p["bits"])
    if kind == "hash":
        return T.Program.gen_hash(p["bits"], p["rounds"])
    if kind == "life":
        return T.Program.gen_life(p["size"], p["size"])
    if kind == "random":
        return T.Program.random(p["cells"], p["len"], p["seed"])
    if kind == "random_in":
        return T.Program.random_in(p["cells"], p["width"], p["len"], p["seed"])
    if kind == "rewrite":
        base = T.Program.random_in(p["cells"], p["width"], p["len"], p["seed"])
        return base.rewrite(p["rseed"], p.get("mutate", False))
    raise ValueError(kind)


def setup(case):
    """Programs, spec and enum arguments of one golden case."""
    a = program(case["a"])
    b = program(case["b"]) if case["mode"] == "equiv" else None
    spec = None
    if case["mode"] != "equiv":
        spec = T.Spec(a, case["spec"], case["mode"] == "verify")
    part = case.get("part", [0, 0, 1])
    kw = dict(ticks=case.get("ticks", 1), part=part[0], part_end=part[1], parts=part[2])
    return MODES[case["mode"]], a, b, spec, kw


def same_result(got, want):
    return (got["space"] == want["space"] and got["tried"] == want["tried"] and
            got["hits"] == want["hits"] and got["hit"] == want["hit"] and
            got["ops"] == want["ops"])


def case_id(c):
    s = c["mode"] + "-" + c["a"]["kind"] + "-" + "-".join(str(v) for v in c["a"]["params"].values())
    if "spec" in c:
        s += "-" + c["spec"].replace(" ", "")
    if "b" in c and c["b"]["params"].get("mutate"):
        s += "-mutated"
    if "part" in c:
        s += "-part" + "_".join(map(str, c["part"]))
    if "ticks" in c:
        s += "-ticks%d" % c["ticks"]
    return s


def random_spec(r, depth: int = 3) -> str:
    """A random right side over a, b and small constants with + - * ^ & | << ~ and negation
    (the spec language's operators), for differential tests of the spec paths."""
    def expr(d):
        if d == 0 or r.random() < 0.25:
            return r.choice(["a", "b", str(r.randrange(1, 9))])
        op = r.choice(["+", "-", "*", "^", "&", "|", "<<", "~", "neg"])
        if op == "~":
            return "~(" + expr(d - 1) + ")"
        if op == "neg":
            return "-(" + expr(d - 1) + ")"
        if op == "<<":
            return "(" + expr(d - 1) + ") << " + str(r.randrange(0, 4))
        return "(" + expr(d - 1) + " " + op + " " + expr(d - 1) + ")"
    return "p = " + ("a * b + " if r.random() < 0.7 else "") + expr(depth)


def load_gz(name):
    import gzip
    with gzip.open(os.path.join(GOLDEN, name), "rt") as f:
        return json.load(f)


def as_record(r):
    """An EnumResult dict in the fixtures' per-job form: [space, tried, hits, ops, "hex,..."]."""
    return [r["space"], r["tried"], r["hits"], r["ops"], ",".join("%x" % x for x in r["hit"])]


def program_digest(s, rename=None) -> str:
    """sha256 of a Program struct's structure by cell names, so that it does not depend on the
    order cells were numbered in: its instructions, id and link cells, inputs and outputs.
    rename maps each cell name first (a listing's spelling of macro-local names)."""
    import hashlib
    names = [s.cell_names[c].decode() for c in range(s.ncells)]
    if rename:
        names = [rename(n) for n in names]
    h = hashlib.sha256()
    h.update(b"%d %d;" % (s.len, s.ncells))
    h.update("".join("%d,%s;" % (s.code[i].op, names[s.code[i].addr])
                     for i in range(s.len)).encode())
    h.update(("in" + ",".join(names[s.inputs[i]] for i in range(s.ninputs))).encode())
    h.update(("out" + ",".join(names[s.outputs[i]] for i in range(s.noutputs))).encode())
    if s.special:
        h.update(("sp" + ";".join(sorted("%s,%d,%d,%s" % (names[c], s.special[c].kind,
                                                        s.special[c].dim,
                                                        names[s.special[c].src])
                                         for c in range(s.ncells)))).encode())
    return h.hexdigest()


def reordered(text: str, seed: int) -> str:
    """The same program with the names of its .in and .out lines in another order.  Cells are
    numbered in declaration order, so its inputs and outputs come in another order; equivalence
    matches them by name (src/enum.c:48-78)."""
    import random
    r = random.Random(seed)
    out = []
    for line in text.splitlines():
        words = line.split()
        if words and words[0] in (".in", ".out"):
            names = words[1:]
            r.shuffle(names)
            line = " ".join([words[0]] + names)
        out.append(line)
    return "\n".join(out) + "\n"


def reordered_pairs():
    """(a, b) equivalence pairs whose second program declares its inputs and outputs in another
    order: identity-rewritten copies (equivalent) and mutated ones, 4 to 12 inputs."""
    pairs = []
    for seed in range(6):
        a = T.Program.random_in(8 + 5 * seed, 4 + seed + seed // 2, 30 + 90 * seed, 5150 + seed)
        for mutate in (False, True):
            b = T.Program.from_asm(reordered(a.rewrite(seed + 40, mutate).text(), seed))
            pairs.append((a, b, mutate))
    return pairs


def with_written_inputs(text: str, k: int) -> str:
    """A random program (every cell an output, src/main.c:1028-1069) with its first k cells made
    inputs, which its stores then overwrite: each pass starts from the assignment, and later
    reads see what the program stored (src/enum.c:115-133)."""
    out, first = [], True
    for line in text.splitlines():
        words = line.split()
        if first and words and words[0] == ".out":  # the first line lists c0 .. c15
            assert len(words) > k + 1
            out.append(" ".join([".in"] + words[1:k + 1]))
            line = " ".join([".out"] + words[k + 1:])
            first = False
        out.append(line)
    return "\n".join(out) + "\n"


def written_input_jobs():
    """(mode, a, b, spec text, ticks) jobs over random programs that store into their inputs:
    equivalence with rewritten and mutated copies and searches for one output, 3 to 12 inputs,
    ticks 1 and 2."""
    jobs = []
    for seed in range(6):
        cells, k = 8 + 6 * seed, 3 + (seed * 7) % 10
        a = T.Program.from_asm(with_written_inputs(
            T.Program.random(cells, 200 + 250 * seed, 9100 + seed).text(), k))
        for ticks in (1, 2):
            for mutate in (False, True):
                jobs.append((T.EN_EQUIV, a, a.rewrite(seed + 7, mutate), None, ticks))
            jobs.append((T.EN_SEARCH, a, None, "c%d = %d" % (k, seed % 2), ticks))
    return jobs
