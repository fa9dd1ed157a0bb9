"""Random cube programs for the cube tests (tests/test_cube_gpu.py on the GPU, tests/test_cube_plan.py
on the CPU)."""
import random


def random_link_program(seed: int, dims: int, cells: int, links: int, length: int) -> str:
    """A random program over plain, id and link cells reaching dimensions below `dims`
    (the shape of tests/test_cube.c:198-241, from Python's own generator)."""
    rnd = random.Random(seed)
    names = ["c%d" % i for i in range(cells)]
    lines = [".out " + " ".join(names[: min(cells, 16)])]
    readable = list(names) + ["ZERO", "ONE"] + ["ID%d" % d for d in range(dims)]
    for i in range(links):
        src = rnd.choice(readable)
        d = rnd.randrange(dims)
        if i == 0:
            d = dims - 1  # the cube spans exactly `dims` dimensions
        lines.append(".link l%d = %s @ %d" % (i, src, d))
        readable.append("l%d" % i)
    for _ in range(length):
        if rnd.random() < 0.6:
            lines.append("NAND " + rnd.choice(readable))
        else:
            lines.append("STO " + rnd.choice(names))
    return "\n".join(lines) + "\n"


def big_random_program(seed: int):
    """A random program over plain, id and link cells built as a struct, the shape of
    tests/test_cube.c:934-1000: 1,024 to 4,096 machines, half of the links to other groups,
    links to links, an eighth of the stores to read-only cells (constants, ids, links), which
    every engine ignores.  The assembler refuses such stores, so the struct is filled directly;
    the returned Program keeps its arrays alive."""
    import ctypes as C
    import tesseract_gb300 as T
    rnd = random.Random(seed)
    dims = 10 + rnd.randrange(3)
    plain, ids, links = 1 + rnd.randrange(20), rnd.randrange(4), 1 + rnd.randrange(16)
    n = 2 + plain + ids + links
    special = (T.CellInfo * n)()
    c = 2 + plain
    for _ in range(ids):
        special[c].kind, special[c].dim = 1, rnd.randrange(dims)
        c += 1
    for _ in range(links):
        special[c].kind = 2
        special[c].dim = 9 + rnd.randrange(dims - 9) if rnd.random() < 0.5 else rnd.randrange(9)
        special[c].src = rnd.randrange(c)
        c += 1
    special[n - 1].kind, special[n - 1].dim = 2, dims - 1  # the cube is that big
    length = 1 + rnd.randrange(120)
    code = (T.Instr * length)()
    for i in range(length):
        code[i].op = rnd.randrange(2)
        a = rnd.randrange(n)
        if code[i].op == 1 and rnd.randrange(8):
            a = 2 + rnd.randrange(plain)
        code[i].addr = a
    names = (C.c_char_p * n)(*[b"ZERO", b"ONE"] + [("c%d" % i).encode() for i in range(2, n)])
    p = T.Program()
    p.s.code, p.s.len, p.s.ncells = code, length, n
    p.s.cell_names, p.s.special = names, special
    p._keep = (code, names, special)  # the struct points into these
    return p, dims
