"""The big-cube demo programs (tc_gen_cube_any / rank / sort, the demos of src/cubedemo.c:398-548)
run on the oracle's reference machine (a lockstep cube, one byte per cell) and checked against
plain Python: OR over all machines, prefix counts, a sorted array.  No GPU: this pins the
generators; tests/test_cubedemo_gpu.py runs the same programs on the GPU cube."""
import random

import pytest

import oracle as O
import tesseract_gb300 as T


def cells(p, stem, n):
    names = [p.s.cell_names[c].decode() for c in range(p.s.ncells)]
    return [names.index("%s%d" % (stem, i)) for i in range(n)]


def cell(p, name):
    names = [p.s.cell_names[c].decode() for c in range(p.s.ncells)]
    return names.index(name)


def run(p, dims, setup):
    n = 1 << dims
    cube = O.RefCube(p, n)
    setup(cube)
    cube.tick()
    return cube


@pytest.mark.parametrize("dims,one", [(9, 0), (9, 300), (9, 2000), (10, 1023)])
def test_any(dims, one):
    p = T.Program.gen_cube_demo("any", dims)
    x, r = cell(p, "x"), cell(p, "r")
    n = 1 << dims
    cube = run(p, dims, lambda c: [c.set(k, x, int(k == one)) for k in range(n)])
    assert all(cube.get(k, r) == int(one < n) for k in range(n))


@pytest.mark.parametrize("dims,seed", [(9, 1), (10, 2)])
def test_rank(dims, seed):
    p = T.Program.gen_cube_demo("rank", dims)
    rnd = random.Random(seed)
    n = 1 << dims
    xs = [int(rnd.random() < 0.3) for _ in range(n)]
    x, pv, tv = cell(p, "x"), cells(p, "p", dims + 1), cells(p, "t", dims + 1)
    cube = run(p, dims, lambda c: [c.set(k, x, xs[k]) for k in range(n)])
    get = lambda k, cs: sum(cube.get(k, c) << i for i, c in enumerate(cs))
    total = sum(xs)
    for k in range(n):
        assert get(k, pv) == sum(xs[:k]) and get(k, tv) == total


@pytest.mark.parametrize("dims,seed", [(9, 3), (10, 4)])
def test_sort(dims, seed):
    p = T.Program.gen_cube_demo("sort", dims)
    rnd = random.Random(seed)
    n = 1 << dims
    vs = [rnd.randrange(256) for _ in range(n)]
    v = cells(p, "v", 8)

    def setup(c):
        for k in range(n):
            for b in range(8):
                c.set(k, v[b], (vs[k] >> b) & 1)

    cube = run(p, dims, setup)
    got = [sum(cube.get(k, v[b]) << b for b in range(8)) for k in range(n)]
    assert got == sorted(vs)


def test_sizes():
    """The programs grow as the algorithms say: dims OR steps, dims add steps, and
    dims (dims + 1) / 2 compare-exchange rounds."""
    for d in (9, 12, 16):
        assert T.Program.gen_cube_demo("any", d).dims() == d
        assert T.Program.gen_cube_demo("rank", d).dims() == d
        s = T.Program.gen_cube_demo("sort", d)
        assert s.dims() == d
        assert len(s) > d * (d + 1) // 2 * 200


@pytest.mark.parametrize("dims,seed", [(9, 5), (10, 6)])
def test_max(dims, seed):
    p = T.Program.gen_cube_demo("max", dims)
    rnd = random.Random(seed)
    n = 1 << dims
    vs = [rnd.randrange(256) for _ in range(n)]
    v, m = cells(p, "v", 8), cells(p, "m", 8)

    def setup(c):
        for k in range(n):
            for b in range(8):
                c.set(k, v[b], (vs[k] >> b) & 1)

    cube = run(p, dims, setup)
    assert all(sum(cube.get(k, m[b]) << b for b in range(8)) == max(vs) for k in range(n))


def mobius(a):
    a = list(a)
    d = 1
    while d < len(a):
        for k in range(len(a)):
            if k & d:
                a[k] ^= a[k ^ d]
        d <<= 1
    return a


@pytest.mark.parametrize("dims,seed", [(9, 7), (10, 8)])
def test_anf_and_walsh(dims, seed):
    rnd = random.Random(seed)
    n = 1 << dims
    fs = [rnd.randrange(2) for _ in range(n)]
    p = T.Program.gen_cube_demo("anf", dims)
    f = cell(p, "f")
    cube = run(p, dims, lambda c: [c.set(k, f, fs[k]) for k in range(n)])
    assert [cube.get(k, f) for k in range(n)] == mobius(fs)
    p = T.Program.gen_cube_demo("walsh", dims)
    f, w = cell(p, "f"), cells(p, "w", dims + 3)
    cube = run(p, dims, lambda c: [c.set(k, f, fs[k]) for k in range(n)])
    mask = (1 << (dims + 3)) - 1
    for k in (0, 1, 5, n // 3, n - 1):
        want = sum((-1) ** (fs[j] ^ (bin(j & k).count("1") & 1)) for j in range(n))
        assert sum(cube.get(k, w[b]) << b for b in range(dims + 3)) == want & mask


@pytest.mark.parametrize("dims,seed", [(9, 9), (11, 10)])
def test_ring(dims, seed):
    p = T.Program.gen_cube_demo("ring", dims)
    rnd = random.Random(seed)
    n = 1 << dims
    xs = [rnd.randrange(2) for _ in range(n)]
    x = cell(p, "x")
    cube = run(p, dims, lambda c: [c.set(k, x, xs[k]) for k in range(n)])
    gray = lambda i: i ^ (i >> 1)
    for i in range(n):
        l, c, r = gray((i - 1) % n), gray(i), gray((i + 1) % n)
        assert cube.get(c, x) == (110 >> ((xs[l] << 2) | (xs[c] << 1) | xs[r])) & 1


def test_polymul_ntt():
    """c = a b in Z_12289[x]/(x^512 + 1) by the NTT program on the reference machine's cube,
    its twiddles computed here from the textbook definition, against the schoolbook product."""
    dims, q, R = 9, 12289, (1 << 14) % 12289
    n = 1 << dims
    p = T.Program.gen_cube_demo("polymul", dims)
    g = 2
    while pow(g, (q - 1) // 2, q) == 1 or pow(g, (q - 1) // 3, q) == 1:
        g += 1
    psi = pow(g, (q - 1) // (2 * n), q)
    rnd = random.Random(11)
    x = [rnd.randrange(q) for _ in range(n)]
    y = [rnd.randrange(q) for _ in range(n)]
    a, b, c = cells(p, "a", 14), cells(p, "b", 14), cells(p, "c", 14)
    zf = [cells(p, "zf%d_" % d, 14) for d in range(dims)]
    zi = [cells(p, "zi%d_" % d, 14) for d in range(dims)]

    def brv(i):
        return int(format(i, "0%db" % dims)[::-1], 2)

    def setup(cube):
        for k in range(n):
            vals = [(a, x[k]), (b, y[k])]
            for d in range(dims):
                zeta = pow(psi, brv((1 << (dims - 1 - d)) + (k >> (d + 1))), q)
                vals.append((zf[d], zeta * R % q))
                vals.append((zi[d], pow(zeta, q - 2, q) * R % q if (k >> d) & 1 else R))
            for cs, v in vals:
                for i, cl in enumerate(cs):
                    cube.set(k, cl, (v >> i) & 1)

    cube = run(p, dims, setup)
    want = [0] * n
    for i in range(n):
        for j in range(n):
            t = x[i] * y[j] % q
            want[(i + j) % n] = (want[(i + j) % n] + (t if i + j < n else q - t)) % q
    got = [sum(cube.get(k, cl) << i for i, cl in enumerate(c)) for k in range(n)]
    assert got == want


@pytest.mark.parametrize("dims,seed,rate", [(9, 12, 0.1), (10, 13, 0.5), (9, 14, 0.0),
                                            (9, 15, 1.0)])
def test_pack(dims, seed, rate):
    """The bytes of the machines with a hit end, in machine order, in the first machines, which
    alone keep h = 1 (src/cubedemo.c:134-151); no hit and every machine a hit included."""
    p = T.Program.gen_cube_demo("pack", dims)
    rnd = random.Random(seed)
    n = 1 << dims
    vs = [rnd.randrange(256) for _ in range(n)]
    hs = [int(rnd.random() < rate) for _ in range(n)]
    v, h = cells(p, "v", 8), cell(p, "h")

    def setup(c):
        for k in range(n):
            c.set(k, h, hs[k])
            for b in range(8):
                c.set(k, v[b], (vs[k] >> b) & 1)

    cube = run(p, dims, setup)
    hits = [x for x, hit in zip(vs, hs) if hit]
    for k in range(n):
        assert cube.get(k, h) == int(k < len(hits))
        if k < len(hits):
            assert sum(cube.get(k, v[b]) << b for b in range(8)) == hits[k]


@pytest.mark.parametrize("dims,seed", [(9, 16), (10, 17)])
def test_xorconv(dims, seed):
    """h(k) = #j with f(j) = g(j ^ k) = 1 (src/cubedemo.c:231-251), against the sum itself."""
    p = T.Program.gen_cube_demo("xorconv", dims)
    rnd = random.Random(seed)
    n = 1 << dims
    fs = [rnd.randrange(2) for _ in range(n)]
    gs = [int(rnd.random() < 0.7) for _ in range(n)]
    f, g, h = cell(p, "f"), cell(p, "g"), cells(p, "h", dims + 1)
    cube = run(p, dims, lambda c: [(c.set(k, f, fs[k]), c.set(k, g, gs[k])) for k in range(n)])
    for k in range(n):
        want = sum(fs[j] & gs[j ^ k] for j in range(n))
        assert sum(cube.get(k, h[b]) << b for b in range(dims + 1)) == want


def test_xorconv_largest_value():
    """f = g = 1 everywhere: h = 2^dims in every machine, the top bit of the dims + 1."""
    dims = 9
    p = T.Program.gen_cube_demo("xorconv", dims)
    f, g, h = cell(p, "f"), cell(p, "g"), cells(p, "h", dims + 1)
    cube = run(p, dims, lambda c: [(c.set(k, f, 1), c.set(k, g, 1)) for k in range(1 << dims)])
    assert all(sum(cube.get(k, h[b]) << b for b in range(dims + 1)) == 1 << dims
               for k in range(1 << dims))
