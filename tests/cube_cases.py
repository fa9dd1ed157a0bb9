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
