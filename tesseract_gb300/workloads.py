"""The benchmark workloads beyond the headline verify, built from the engine's own generators.

serve_stream       a Poisson stream (mean `rate` jobs/s, seed 1) of mixed jobs: verify of
                   `gen mul` multipliers (8..16 bits) against p = a * b; equivalence of random
                   programs with inputs (100..20,000 instructions log-uniform, 16..34 input bits,
                   8..64 cells) against their rewritten copies; search of such programs for every
                   input whose outputs equal a random target.

batch_equiv_jobs   4,096 random programs with inputs (seeds 0..4095; cells uniform 8..64;
                   length log-uniform 16..4,096; input width uniform 16..28), each paired with a
                   copy rewritten by local NAND identities; every `mutate_every`-th pair is a
                   negative control whose last STO became a NAND.  The parameters of job s come
                   from splitmix64(s).
"""
from __future__ import annotations

import tesseract_gb300 as T

M64 = (1 << 64) - 1


def splitmix64(state: int):
    state = (state + 0x9E3779B97F4A7C15) & M64
    z = state
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
    return state, z ^ (z >> 31)


def job_shape(seed: int):
    """(cells, width, length) of batch job `seed`."""
    s = seed * 0x2545F4914F6CDD1D & M64
    s, r1 = splitmix64(s)
    s, r2 = splitmix64(s)
    s, r3 = splitmix64(s)
    cells = 8 + r1 % 57
    width = 16 + r2 % 13
    u = (r3 >> 11) / float(1 << 53)
    length = int(round(16 * 256 ** u))
    return cells, width, max(16, min(4096, length))


def batch_equiv_jobs(n: int = 4096, mutate_every: int = 8, width_cap: int | None = None,
                     seeds=None):
    """The batch's jobs for seeds 0..n-1, or for the given seeds (same generator and shapes)."""
    jobs = []
    for seed in (range(n) if seeds is None else seeds):
        cells, width, length = job_shape(seed)
        if width_cap:
            width = min(width, width_cap)
        a = T.Program.random_in(cells, width, length, seed)
        b = a.rewrite(seed, mutate=(seed % mutate_every) == mutate_every - 1)
        jobs.append(dict(mode=T.EN_EQUIV, a=a, b=b, ticks=1, seed=seed,
                         mutated=(seed % mutate_every) == mutate_every - 1))
    return jobs


def serve_stream(n: int = 512, rate: float = 2000.0, seed: int = 1, max_width: int = 34,
                 min_width: int = 16):
    """(jobs, arrival times): the serving workload."""
    import math
    state = (seed * 0x9E3779B97F4A7C15) & M64
    def rnd():
        nonlocal state
        state, z = splitmix64(state)
        return z
    def uniform():
        return (rnd() >> 11) / float(1 << 53)
    jobs, arrivals, t = [], [], 0.0
    muls = {}
    for i in range(n):
        t += -math.log(1.0 - uniform()) / rate
        arrivals.append(t)
        kind = rnd() % 5
        if kind == 0:
            bits = 8 + rnd() % 9
            if bits not in muls:
                muls[bits] = T.Program.gen_mul(bits)
            p = muls[bits]
            jobs.append(dict(mode=T.EN_VERIFY, a=p, spec=T.Spec(p, "p = a * b"), kind="verify",
                             bits=bits))
            continue
        cells = 8 + rnd() % 57
        width = min_width + rnd() % (max_width - min_width + 1)
        length = int(round(100 * 200 ** uniform()))
        a = T.Program.random_in(cells, width, length, 1000000 + i)
        if kind in (1, 2):
            b = a.rewrite(i, mutate=(rnd() % 4 == 0))
            jobs.append(dict(mode=T.EN_EQUIV, a=a, b=b, kind="equiv", width=width))
        else:
            target = rnd() & ((1 << cells) - 1)
            spec = T.Spec(a, "c = %d" % target, False)
            jobs.append(dict(mode=T.EN_SEARCH, a=a, spec=spec, kind="search", width=width))
    return jobs, arrivals
