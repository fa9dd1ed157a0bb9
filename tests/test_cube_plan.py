"""The cube's plan, on the CPU.

Far reads of computed cells: where the value read is a function of cells the segment never
writes, the reading warp computes it again for the other machine instead of cutting the pass
(tesseract_gb300/csrc/cube.c, find_cuts_recompute); the generated kernels of such plans compile
for sm_103a (nvcc), and the GPU tests check them against the reference machine.

Closing copies: a pass's closing copies (A <- B: a Life board taking its next generation from the
cells it was computed into) are left out of every pass of a cube run but the last: the engine compiles its
kernels twice, the second time with A's and B's memory exchanged, and alternates.  That is sound
when the copies are plain (every B copied to one A, no B written and no A read among them), the
pass begins by setting RR, and every B is written before it is read, so that what a pass finds in
B's memory is never seen (tesseract_gb300/csrc/cube.c, copy_tail).

No GPU: the plan the engine makes (tc_cube_copy_plan) is applied on the oracle's reference
machine, where running a pass in the other memory variant is the same as exchanging A's and B's
values before it, and the state after several passes must equal the plain run's, cell by cell and
RR, in every machine.  Programs that break a condition get no plan."""
import ctypes as C
import os
import random
import shutil
import subprocess
import tempfile

import pytest

import oracle as O
import tesseract_gb300 as T
from cube_cases import random_link_program

NVCC = shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc"
                                if os.path.exists("/usr/local/cuda/bin/nvcc") else None)


def cube_source(p, variant=0, recompute=True):
    """(kernels per pass, the source of the pass's kernels in memory variant `variant`)."""
    L = T.lib()
    L.tc_cube_source.restype = C.c_void_p
    L.tc_cube_source.argtypes = [C.c_void_p, C.c_uint, C.POINTER(C.c_uint),
                                 C.POINTER(C.c_size_t)]
    flag = C.c_int.in_dll(L, "tc_cube_recompute")
    old, flag.value = flag.value, int(recompute)
    try:
        nk, n = C.c_uint(), C.c_size_t()
        ptr = L.tc_cube_source(p.ptr, variant, C.byref(nk), C.byref(n))
    finally:
        flag.value = old
    if not ptr:
        return nk.value, None
    text = C.string_at(ptr, n.value).decode()
    C.CDLL(None).free(C.c_void_p(ptr))
    return nk.value, text


def recomputing_programs(count, dims):
    """Seeded random link programs whose plan recomputes at least one far read."""
    out, seed = [], 0
    while len(out) < count:
        text = random_link_program(seed, dims, 24, 24, 400)
        p = T.Program.from_asm(text)
        if cube_source(p, recompute=True)[0] < cube_source(p, recompute=False)[0]:
            out.append((seed, text))
        seed += 1
    return out


def plan(p):
    L = T.lib()
    L.tc_cube_copy_plan.restype = C.c_int
    L.tc_cube_copy_plan.argtypes = [C.c_void_p, C.POINTER(C.c_size_t), C.POINTER(C.c_uint32)]
    slot = (C.c_uint32 * (p.s.ncells + 1))()
    start = C.c_size_t()
    if not L.tc_cube_copy_plan(p.ptr, C.byref(start), slot):
        return None
    pairs = [(a, slot[a]) for a in range(p.s.ncells) if slot[a] > a]
    return start.value, pairs


def plain_cells(p):
    """Cells a random state may fill: not ZERO/ONE, not id or link cells."""
    out = []
    for c in range(2, p.s.ncells):
        if p.s.special and p.s.special[c].kind != 0:
            continue
        out.append(c)
    return out


def random_cube(p, machines, seed):
    cube = O.RefCube(p, machines)
    rnd = random.Random(seed)
    for k in range(machines):
        for c in plain_cells(p):
            cube.set(k, c, rnd.randrange(2))
        cube.set_rr(k, rnd.randrange(2))
    return cube


def state(cube, p, machines):
    cells = plain_cells(p)
    return [[cube.get(k, c) for c in cells] + [cube.rr(k)] for k in range(machines)]


def run_exchanged(p, cube, machines, passes, start, pairs):
    """Every pass but the last without its closing copies (their effect on A and RR undone), A's
    and B's values exchanged after it, as the other memory variant sees them."""
    for i in range(passes):
        if i + 1 == passes:
            cube.tick()
            break
        for _ in range(start):
            cube.step()
        keep = [([cube.get(k, a) for a, _ in pairs], cube.rr(k)) for k in range(machines)]
        for _ in range(len(p) - start):
            cube.step()
        for k in range(machines):
            vals, rr = keep[k]
            cube.set_rr(k, rr)
            for (a, b), v in zip(pairs, vals):
                cube.set(k, a, v)                # the pass without its copies ...
            for a, b in pairs:                   # ... and the other variant's view of it
                va, vb = cube.get(k, a), cube.get(k, b)
                cube.set(k, a, vb)
                cube.set(k, b, va)


@pytest.mark.parametrize("passes", [1, 2, 3, 4])
def test_life_board_copies_exchanged_match_the_plain_run(passes):
    p = T.Program.gen_life_cube(4, 4, 5, 6)  # 2,048 machines: far reads, three segments
    machines = 1 << p.dims()
    got = plan(p)
    assert got is not None
    start, pairs = got
    assert len(pairs) == 16 and start < len(p)
    plain = random_cube(p, machines, 7)
    for _ in range(passes):
        plain.tick()
    other = random_cube(p, machines, 7)
    run_exchanged(p, other, machines, passes, start, pairs)
    assert state(other, p, machines) == state(plain, p, machines)


def test_plan_of_the_full_life_board():
    """gen_life_cube(32, 32, 8, 8): 1,024 board cells take their next generation in the last
    segment (4,096 instructions)."""
    p = T.Program.gen_life_cube(32, 32, 8, 8)
    start, pairs = plan(p)
    assert len(pairs) == 1024 and len(p) - start == 4096


BASE = (".in x\n.out x\n.link lx = x @ 10\n"
        "NAND ZERO\nNAND lx\nSTO y\n")          # y from x across dimension 10
COPY = "NAND ZERO\nNAND y\nNAND ONE\nSTO x\n"  # x <- y after x was read far: a new segment


def test_small_program_gets_a_plan():
    p = T.Program.from_asm(BASE + COPY)
    assert plan(p) is not None


@pytest.mark.parametrize("text", [
    ".in x\n.out x\n.link lx = x @ 10\nNAND ZERO\nNAND y\nSTO z\nNAND lx\nSTO y\n" + COPY,  # y read first
    ".in x\n.out x\n.link lx = x @ 10\nNAND ONE\nNAND lx\nSTO y\n" + COPY,  # RR live at the start
    BASE + "NAND ZERO\nNAND y\nSTO x\n",                                    # a NOT, not a copy
    BASE + "NAND ZERO\nNAND y\nNAND ONE\nSTO x\nSTO w\n",                    # one B, two As
    BASE + "NAND ZERO\nNAND y\nNAND ONE\nSTO x\nNAND ZERO\nNAND x\nNAND ONE\nSTO w\n",  # A read
])
def test_unsound_programs_get_no_plan(text):
    p = T.Program.from_asm(text)
    assert plan(p) is None


def test_life_is_one_kernel_per_generation():
    """gen_life_cube(32, 32, 8, 8): the west and east halo cells the north and south halos read
    across far dimensions are recomputed, so the masks, the halos and the rule are one kernel;
    the closing copies are the other (run only at the end of a run).  Without recomputation:
    three."""
    p = T.Program.gen_life_cube(32, 32, 8, 8)
    assert cube_source(p, recompute=True)[0] == 2
    assert cube_source(p, recompute=False)[0] == 3


@pytest.mark.skipif(NVCC is None, reason="nvcc not installed")
@pytest.mark.parametrize("which", ["life", "random"])
def test_recomputing_kernels_compile(which):
    if which == "life":
        progs = [T.Program.gen_life_cube(4, 4, 5, 6)]
    else:
        progs = [T.Program.from_asm(t) for _, t in recomputing_programs(3, 13)]
    d = tempfile.mkdtemp()
    for i, p in enumerate(progs):
        for variant in (0, 1):
            nk, src = cube_source(p, variant)
            if src is None:
                continue
            assert "#error" not in src
            path = os.path.join(d, "cube%d_%d.cu" % (i, variant))
            with open(path, "w") as f:
                f.write(src)
            r = subprocess.run([NVCC, "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17",
                                "-Xptxas", "-O2", "-c", path, "-o", path + ".o"],
                               capture_output=True, text=True, timeout=600)
            assert r.returncode == 0, r.stderr[-2000:]


def test_recomputing_never_adds_kernels():
    """On random link programs over 1,024 to 8,192 machines, recomputing far reads only ever
    removes cuts: never more kernels than the plain rule."""
    fewer = 0
    for seed in range(40):
        text = random_link_program(500 + seed, 10 + seed % 4, 20, 16, 300)
        p = T.Program.from_asm(text)
        with_rc, plain = cube_source(p, recompute=True)[0], cube_source(p, recompute=False)[0]
        assert with_rc <= plain, seed
        fewer += with_rc < plain
    assert fewer > 0  # the programs do exercise it


def kernel_lop3(src):
    """LOP3 count of each kernel in a pass's source."""
    return [k.count("TC_LOP3(") for k in src.split('extern "C" __global__')[1:]]


def test_recomputing_stays_within_its_budget():
    """The NTT product on 2,048 machines: recomputing every far read it could would put most of
    the pass into one kernel that cannot be split (400,000 LOP3, minutes of compiling); the
    per-segment budget cuts instead, so no kernel is much larger than the plain rule's largest
    (the small recomputations the budget allows add a few LOP3).  Life's
    recomputations fit the budget (one kernel per generation, the test above)."""
    p = T.Program.gen_cube_demo("polymul", 11)
    _, with_rc = cube_source(p, recompute=True)
    _, plain = cube_source(p, recompute=False)
    assert max(kernel_lop3(with_rc)) <= 1.05 * max(kernel_lop3(plain))
    L = T.lib()
    budget = C.c_int.in_dll(L, "tc_cube_recompute_budget")
    old, budget.value = budget.value, 1 << 30
    try:
        _, unbounded = cube_source(p, recompute=True)
    finally:
        budget.value = old
    assert max(kernel_lop3(unbounded)) > 2 * max(kernel_lop3(plain))  # what the budget prevents


def test_long_segments_split_into_equal_kernels():
    """A segment longer than one kernel may hold (140,000 instructions) is split into equal
    kernels of at most 50,000, which compile in parallel: the NTT product on 512 machines (one
    segment of 272,001) becomes 6 kernels.  Life on 512 machines (130,575) stays one kernel, so
    its passes still loop inside it."""
    p = T.Program.gen_cube_demo("polymul", 9)
    assert p.s.len == 272001
    assert cube_source(p)[0] == 6
    life = T.Program.gen_life_cube(32, 32, 4, 5)
    assert cube_source(life)[0] == 1
