"""Benchmark: exhaustive verify of the 16 x 16 array multiplier on the GPU, and the other
workloads beside it.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--config verify|life|batch|super|serve] [--replicas]

Headline workload (one step): `alpha verify <gen mul --bits 16> --spec "p = a * b"` -- the
6,040-instruction NAND/STO multiplier run on all 2^32 (a, b) and compared with a * b, through the
engine's C ABI (cuda_enum_run).  The metric is the reference's "1-bit operations" (program length
x assignments x ticks, src/enum.c:164): 6,040 x 2^32 = 2.594e13 lane-ops per step.

  value      lane-ops/s from the kernel's own CUDA-event time (device work only); beside it
             assignments/s
  e2e        lane-ops/s from the host clock around the C-ABI call: code generation and module
             cache lookup, launch, and the device-to-host read of the result
  roofline   the verify kernel against the measured LOP3 issue rate of the same GPU
             (cuda_lop3_peak, 32-bit 3-input logic ops/s): achieved = the logic operations the
             generated kernel issues per 32-lane word (LUTs per step, hoisted LUTs over their
             stretch, the compare's carry chain; counted by the code generator) x words / kernel
             time.  frac_accounting is the reference's lane-op accounting over the same peak
             x 32 lanes (above 1: the LUT network and the hoisting do less work than 6,040 NAND/STO
             per lane).
  sustained  the same launch back to back for at least 5 s, with the SM clock sampled
  configs    the other four workloads (cube Life, the 4,096-pair batch, the superoptimizer, the
             served streams), each with its own clocks, wall time and pass/fail
  cpu_baseline  the oracle's CPU port of the reference's enumerator (bit-sliced, all host
             threads, scalar per-lane spec compare as in src/enum.c:186-200) on a bounded sample

--impl reference times the reference's own enumerator where it was built from its sources on
this host (x86), else the oracle's C port of it (the reference's AVX2/x86 engines do not build on
the aarch64 GPU host).  Its inputs are the reference's own generator output
(tests/golden/mul16.asm.gz, sha256-pinned) read by the oracle: nothing of this engine is loaded.

With N > 1 (torchrun, one rank per GPU) rank r verifies share r of N of the space (the
reference's --part rule, no exchange on the data path) and the shares' results are gathered and
merged once afterwards (scaling "strong"); --replicas runs the whole space on every rank
instead (scaling "weak").
"""
from __future__ import annotations

import argparse
import gzip
import hashlib
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")

METRIC = "bit-exact 1-bit NAND lane-ops/s vs LOP3 peak; batched jobs/s, p50/p99 vs plain"
WORKLOAD = ("verify gen mul --bits 16 (6040 NAND/STO instructions, 72 cells) over all 2^32 "
            "(a, b) against p = a * b")

# dram__bytes_read.sum + dram__bytes_write.sum of one full-space tc_enum launch, from the ncu
# capture summarised in this file (the kernel's code and arguments; its state is in registers)
VERIFY_DRAM_BYTES = 32768
VERIFY_PROFILE = "profiles/tc_enum_verify_mul16.md"
VERIFY_ALU_PIPE_NCU = 0.979


def measured_peaks() -> dict:
    """MEASURED_PEAKS.json beside this file, when the run has one."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def dist_env():
    return int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")), \
        int(os.environ.get("LOCAL_RANK", "0"))


class Clocks:
    """nvidia-smi sampled every 200 ms while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int = 0):
        self.gpu = gpu
        self.p = None
        self.out = ""

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" +
                                       self.FIELDS, "--format=csv,noheader,nounits", "-lms",
                                       "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                                      text=True)
        except OSError:
            self.p = None
        return self

    def __exit__(self, *exc):
        if self.p:
            self.p.terminate()
            try:
                self.out, _ = self.p.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.p.kill()

    def summary(self):
        sm, mx, power, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.out.splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
                power.append(float(f[3]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "samples": len(sm),
                "power_w_max": max(power), "reasons": sorted(reasons)}


# ---- the CPU side: the reference's inputs, read by the oracle --------------------------------

def reference_inputs():
    """The headline program and spec without this engine: the text the reference's `gen mul
    --bits 16` printed (tests/golden/mul16.asm.gz, checked against the sha256 pinned in
    tests/golden/programs.json), read by the oracle, and `p = a * b` laid out by the oracle."""
    import oracle as O
    with gzip.open(os.path.join(GOLDEN, "mul16.asm.gz"), "rt") as f:
        text = f.read()
    with open(os.path.join(GOLDEN, "programs.json")) as f:
        pinned = json.load(f)['mul:{"bits": 16}']
    if hashlib.sha256(text.encode()).hexdigest() != pinned:
        raise RuntimeError("tests/golden/mul16.asm.gz is not the reference's gen mul output")
    prog = O.PrintedProgram(text)
    return prog, prog.product_spec()


def cpu_sample(seconds_target=12.0):
    """The oracle's CPU port on a bounded sample of the headline workload: lane-ops/s."""
    import oracle as O
    prog, spec = reference_inputs()
    e = O.verify_struct(prog, spec)
    threads = os.cpu_count() or 1
    chunks = threads
    while True:
        t0 = time.perf_counter()
        r = O.enum_run_struct(e, threads=threads, limit_chunks=chunks)
        dt = time.perf_counter() - t0
        if dt > seconds_target / 4 or chunks > 1 << 20:
            break
        chunks *= 4
    if dt < seconds_target * 0.8:
        chunks = max(chunks, int(chunks * seconds_target / dt))
        t0 = time.perf_counter()
        r = O.enum_run_struct(e, threads=threads, limit_chunks=chunks)
        dt = time.perf_counter() - t0
    assert r["hits"] == 0
    return {"value": r["ops"] / dt, "unit": "lane-ops/s", "cores": threads, "kind": "port",
            "sample": f"{chunks} chunks of 32768 assignments ({r['tried']} of 2^32), "
                      f"{dt:.1f} s, 0 mismatches"}, r, dt


def run_reference(args):
    """The reference arm: the reference's own enumerator where it was built from its sources on
    this host (oracle/_ref/alpha, x86 only: `alpha verify ... --part i/K --raw`, a 1/K share of
    the space per step, K = 64 for up to 100 steps and more beyond), otherwise the oracle's C port
    of it on every host core on a sample of chunks sized per step; either way the whole run takes
    about two minutes."""
    world, rank, _ = dist_env()
    if rank != 0:
        return 0
    import oracle as O
    threads = os.cpu_count() or 1
    # each step is a bounded sample, sized so that all warm-up and timed steps take about two
    # minutes whatever --steps is (at most 4 s a step)
    nsteps = args.steps + args.warmup
    per_step_s = min(4.0, 120.0 / max(1, nsteps))
    if O.have_reference():
        import tempfile
        parts = 64 * max(1, -(-nsteps // 100))  # a share of 2^32 / parts assignments per step
        with tempfile.TemporaryDirectory() as d:
            prog = os.path.join(d, "mul16.asm")
            with open(prog, "w") as f:
                f.write(subprocess.run([O.REF_BIN, "gen", "mul", "--bits", "16"], check=True,
                                       capture_output=True, text=True).stdout)

            def step(i):
                out = subprocess.run([O.REF_BIN, "verify", prog, "--spec", "p = a * b", "--part",
                                      "%d/%d" % (i % parts, parts), "--raw"], check=True,
                                     capture_output=True, text=True).stdout
                f = out.split("\n")[0].split()
                assert f[0] == "EN" and int(f[4]) == 0
                return int(f[7])
            for i in range(args.warmup):
                step(i)
            ops = 0
            t0 = time.perf_counter()
            for i in range(args.steps):
                ops += step(args.warmup + i)
            dt = time.perf_counter() - t0
        kind, sample = "reference", ("alpha verify --part i/%d (2^32 / %d assignments) per step"
                                     % (parts, parts))
    else:
        prog, spec = reference_inputs()
        e = O.verify_struct(prog, spec)
        base, _, _ = cpu_sample(seconds_target=4.0)
        chunks = max(threads, int(int(base["sample"].split()[0]) * per_step_s / 4.0))
        for _ in range(args.warmup):
            O.enum_run_struct(e, threads=threads, limit_chunks=max(1, chunks // 8))
        ops = 0
        t0 = time.perf_counter()
        for _ in range(args.steps):
            r = O.enum_run_struct(e, threads=threads, limit_chunks=chunks)
            assert r["hits"] == 0
            ops += r["ops"]
        dt = time.perf_counter() - t0
        kind, sample = "port", f"{chunks} chunks of 32768 assignments per step"
    v = ops / dt
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "lane-ops/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True,
            "scaling": "strong", "vs_baseline": None, "dtype": "u64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "sample_per_step": sample},
            "cpu_baseline": {"value": v, "unit": "lane-ops/s", "cores": threads, "kind": kind,
                             "sample": sample},
            "e2e": {"value": v, "unit": "lane-ops/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    if kind == "port":
        line["note"] = ("the reference's AVX2 lane engine and x86 JIT do not build on this host; "
                        "this is the oracle's portable C port of its enumerator, on the "
                        "reference's own gen mul output")
    print(json.dumps(line), flush=True)
    return 0


# ---- the other workloads ---------------------------------------------------------------------

def config_life(gens=1000):
    """Config 2: one 8192 x 8192 B3/S23 board on 65,536 machines (gen_life_cube 32 x 32 tiles,
    2^8 x 2^8 machines), board from splitmix64(42), `gens` generations on the GPU cube engine,
    checked bit for bit against plain C Life (the oracle's word-parallel life_scalar)."""
    import oracle as O
    import tesseract_gb300 as T
    from tesseract_gb300.life import LifeCube, pack_rows, unpack_rows
    t0 = time.perf_counter()
    L = LifeCube(16)
    setup_s = time.perf_counter() - t0
    L.seed(42)
    t0 = time.perf_counter()
    tune = L.cube.tune(32)  # warps and word runs per group-major block, measured on this board
    tune["seconds"] = time.perf_counter() - t0
    start = L.board()
    L.run(16)                       # warm-up: graph capture, first launches
    L.seed(42)
    with Clocks() as clk:
        t0 = time.perf_counter()
        ms = L.run(gens)
        wall = time.perf_counter() - t0
    final = L.board()
    # the same board for 100 times as many generations back to back (about a second), so the
    # rate is also known under the clock the GPU holds over a longer run
    L.seed(42)
    with Clocks() as clk_long:
        ms_long = L.run(100 * gens)
    packed = pack_rows(start)
    tc = time.perf_counter()
    O.life_words(packed, gens)
    cpu_s = time.perf_counter() - tc
    ok = bool((unpack_rows(packed) == final).all())
    n = L.program
    rec = {"metric": "generations/s (cube Life, 65,536 machines, 8192^2 board)",
           "value": gens / (ms / 1e3), "unit": "gen/s", "gens": gens,
           "bit_exact_vs_plain_c": ok, "kernel_ms": ms, "wall_s": wall,
           "cell_updates_per_s": gens * 8192 * 8192 / (ms / 1e3),
           "lane_ops_per_s": gens * len(n) * 65536 / (ms / 1e3),
           "program": {"instructions": len(n), "cells": n.ncells,
                       "segments": L.cube.segments, "kernels_per_pass": L.cube.kernels,
                       "closing_copy_kernels": L.cube.closing_copies,
                       "kernels_per_generation": L.cube.kernels - L.cube.closing_copies},
           "setup_s_incl_nvrtc": setup_s, "autotune": tune, "cpu_word_parallel_life_s": cpu_s,
           "cpu_threads": os.cpu_count(), "clocks": clk.summary(),
           "sustained": {"gens": 100 * gens, "value": 100 * gens / (ms_long / 1e3),
                         "unit": "gen/s", "kernel_ms": ms_long, "clocks": clk_long.summary()}}
    # the exchange between machines: 1,056 link reads per machine per generation (4 gathers
    # of the tile edges), one bit each, 476 of them across 512-machine groups
    exchange = 65536 * 1056 / 8
    peaks = measured_peaks()
    gbs = exchange * gens / (ms / 1e3) / 1e9
    rec["roofline"] = {"bound": "instruction issue and latency (2,048 words of state per cell; "
                                "the 27.2 MB state stays in L2)",
                       "exchange_bytes_per_gen": exchange, "achieved": gbs,
                       "peak": peaks.get("hbm_gbs"), "unit": "GB/s",
                       "frac": gbs / peaks["hbm_gbs"] if peaks.get("hbm_gbs") else None,
                       "peak_source": "MEASURED_PEAKS.json hbm_gbs (copy bandwidth); the "
                                      "exchange is served from L2, not HBM",
                       "traffic": None}
    return rec, ok


def config_batch(njobs=4096):
    """Config 3: the 4,096 random equivalence pairs (workloads.batch_equiv_jobs) in one call,
    every verdict against the reference's own (tests/golden/batch_equiv.json.gz).  The batch
    runs three times: cold (nothing of it compiled: the interpreter runs the light jobs in one
    persistent launch while the host compiles the heavy ones), again with the kernels the
    first run compiled in the cache, and once more after cuda_batch_prepare has compiled the
    kernel of every job worth a launch (its seconds reported apart).  The plain engine (one NVRTC-compiled kernel per job, in
    order) runs 32 jobs of the same distribution that the batch does not contain (seeds 4096 +
    128 k), compiling and then cached."""
    import tesseract_gb300 as T
    from tesseract_gb300.workloads import batch_equiv_jobs
    jobs = batch_equiv_jobs(njobs)
    T.batch_run(batch_equiv_jobs(seeds=range(100000, 100064)))  # warm-up on other programs
    runs = {}
    prep_s = nprep = None
    with Clocks() as clk:
        for label in ("cold", "cached", "all_kernels_cached"):
            if label == "all_kernels_cached":
                # every job worth a launch compiled and loaded beforehand: the batch against
                # the plain engine with its kernels cached, like for like
                t0 = time.perf_counter()
                nprep = T.batch_prepare(jobs)
                prep_s = time.perf_counter() - t0
            t0 = time.perf_counter()
            res = T.batch_run(jobs)
            wall = time.perf_counter() - t0
            st = T.batch_stats()
            runs[label] = {"jobs_per_s": len(jobs) / wall, "wall_s": wall,
                           "jobs_on_generated_kernels": st["compiled"],
                           "jobs_on_interpreter": st["interpreted"],
                           "compile_threads": st["compile_threads"],
                           "planned_for_generated_kernels": st["planned"],
                           "taken_back_by_interpreter": st["taken_back"],
                           "compile_busy_s": st["compile_busy"],
                           "module_load_s": st["compile_load"],
                           "interpreter_start_s": st["interpreter_start"],
                           "interpreter_end_s": st["interpreter_end"],
                           "compiled_end_s": st["compiled_end"],
                           "lane_ops_per_s": sum(r["ops"] for r in res) / wall,
                           "results": res}
    ref = None
    golden = os.path.join(GOLDEN, "batch_equiv.json.gz")
    if njobs == 4096 and os.path.exists(golden):
        with gzip.open(golden, "rt") as f:
            want = json.load(f)["results"]
        ref = True
        for run in runs.values():
            got = [[r["space"], r["tried"], r["hits"], r["ops"],
                    ",".join("%x" % x for x in r["hit"])] for r in run["results"]]
            ref = ref and got == want
    res = runs["cold"]["results"]
    keys = ("space", "tried", "hits", "hit", "ops")
    same_runs = all(a[k] == b[k] for other in ("cached", "all_kernels_cached")
                    for a, b in zip(runs["cold"]["results"], runs[other]["results"]) for k in keys)
    controls = [r["hits"] for j, r in zip(jobs, res) if j["mutated"]]
    sample = batch_equiv_jobs(seeds=range(4096, 4096 + 32 * 128, 128))
    t0 = time.perf_counter()
    plain = [T.enum_run(j["mode"], j["a"], j["b"]) for j in sample]
    plain_cold = time.perf_counter() - t0
    t0 = time.perf_counter()
    plain2 = [T.enum_run(j["mode"], j["a"], j["b"]) for j in sample]
    plain_warm = time.perf_counter() - t0
    batched = T.batch_run(sample)
    same = all(p["hits"] == q["hits"] == b["hits"] and p["hit"] == q["hit"] == b["hit"]
               for p, q, b in zip(plain, plain2, batched))
    for run in runs.values():
        del run["results"]
    pc, pw = len(sample) / plain_cold, len(sample) / plain_warm
    rate = runs["cold"]["jobs_per_s"]
    rec = {"metric": "batched equivalence jobs/s", "jobs": len(jobs), "value": rate,
           "unit": "jobs/s", "runs": runs, "lane_ops": sum(r["ops"] for r in res),
           "bit_exact_vs_reference": ref, "cold_equals_cached": same_runs,
           "negative_controls": len(controls),
           "negative_controls_detected": sum(1 for h in controls if h),
           "plain_sample_jobs": len(sample),
           "plain_jobs_per_s_with_compile": pc, "plain_jobs_per_s_cached": pw,
           "speedup_vs_plain_with_compile": rate / pc,
           "speedup_cached_vs_plain_cached": runs["cached"]["jobs_per_s"] / pw,
           "prepared_kernels": nprep, "prepare_s": prep_s,
           "speedup_all_kernels_cached_vs_plain_cached":
               runs["all_kernels_cached"]["jobs_per_s"] / pw,
           "sample_batched_identical_to_plain": same, "clocks": clk.summary()}
    return rec, bool(same and same_runs and ref is not False)


def config_super():
    """Config 4: the shortest NAND/STO full adder (19, nothing of 18 or fewer) and XOR (7)."""
    import tesseract_gb300 as T
    out = []
    with Clocks() as clk:
        t0 = time.perf_counter()
        for text, want in (("RR = RR ^ x", 7), ("s{a,b} = a ^ b ^ c; c = a&b | a&c | b&c", 19)):
            t1 = time.perf_counter()
            r = T.super_search(text, max_cost=24, quiet=True)
            out.append({"spec": text, "cost": r["cost"], "below": r["below"], "expected": want,
                        "nodes": r["nodes"], "seconds": time.perf_counter() - t1,
                        "checked": r["checked"],
                        "program": [" ".join(x) for x in r["program"]]})
        wall = time.perf_counter() - t0
    ok = all(x["cost"] == x["expected"] == x["below"] and x["checked"] for x in out)
    rec = {"metric": "proven shortest programs", "value": out[-1]["seconds"], "unit": "s",
           "higher_is_better": False, "results": out, "wall_s": wall, "clocks": clk.summary(),
           "reference_here": "alpha super FA: 19, nothing <= 18, 1.2e10 nodes, 87.2 s on 8 x86 "
                             "threads"}
    return rec, ok


def config_serve(n=400):
    """Config 5: a Poisson stream (2,000 jobs/s, seed 1) of mixed verify / equiv / search jobs,
    served with continuous batching (interpreter waves and compiled kernels, routed per job);
    p50/p99 latency and jobs/s, every result against the reference's own
    (tests/golden/serve_stream.json.gz), and the plain engine (one NVRTC-compiled kernel per
    job, in arrival order) on the first jobs of the same stream, timed before serving so that
    their compilation counts."""
    import tesseract_gb300 as T
    from tesseract_gb300.workloads import serve_stream
    golden = os.path.join(GOLDEN, "serve_stream.json.gz")
    want = None
    if n == 400 and os.path.exists(golden):
        with gzip.open(golden, "rt") as f:
            want = json.load(f)["streams"]
    lines, ok = [], True
    for wmax in (34, 22):
        jobs, arrivals = serve_stream(n, rate=2000.0, seed=1, max_width=wmax)
        sample = jobs[:16]
        t0 = time.perf_counter()
        plain = [T.enum_run(j["mode"], j["a"], j.get("b"), j.get("spec")) for j in sample]
        plain_s = time.perf_counter() - t0
        T.serve_run(sample[:4], [0.0] * 4)  # warm-up: streams, slots, threads
        engines = []
        with Clocks() as clk:
            t0 = time.perf_counter()
            res, start, finish = T.serve_run(jobs, arrivals, engines=engines)
            wall = time.perf_counter() - t0
        same = all(p[k] == r[k] for p, r in zip(plain, res)
                   for k in ("space", "tried", "hits", "hit", "ops"))
        ref = None
        if want:
            got = [[r["space"], r["tried"], r["hits"], r["ops"],
                    ",".join("%x" % x for x in r["hit"])] for r in res]
            ref = got == want[str(wmax)]
        ok = ok and same and ref is not False
        lat = sorted(f - a for f, a in zip(finish, arrivals))
        ops = sum(r["ops"] for r in res)
        q = lambda p: lat[min(len(lat) - 1, int(p * len(lat)))]
        span = max(finish) - min(arrivals)
        plain_rate = len(sample) / plain_s
        lines.append({"jobs": n, "max_width": wmax, "offered_jobs_per_s": 2000.0,
                      "value": n / span, "unit": "jobs/s", "p50_s": q(0.50), "p99_s": q(0.99),
                      "wall_s": wall, "jobs_on_generated_kernels": sum(engines),
                      "lane_ops": ops, "lane_ops_per_s": ops / span,
                      "offered_lane_ops_per_s": ops / (arrivals[-1] - arrivals[0]),
                      "bit_exact_vs_reference": ref, "plain_sample_jobs": len(sample),
                      "plain_jobs_per_s_with_compile": plain_rate,
                      "served_vs_plain": (n / span) / plain_rate,
                      "sample_identical_to_plain": same, "clocks": clk.summary()})
    return {"metric": "served jobs/s, p50/p99 latency", "streams": lines}, ok


CONFIGS = {"life": config_life, "batch": config_batch, "super": config_super,
           "serve": config_serve}


def run_configs(names):
    """Each named workload with its own pass/fail and wall time; an error is recorded, not
    raised, so that the headline line is still printed."""
    out = {}
    for name in names:
        t0 = time.perf_counter()
        try:
            rec, ok = CONFIGS[name]()
        except Exception as e:  # noqa: BLE001 -- reported in the line
            rec, ok = {"error": "%s: %s" % (type(e).__name__, e)}, False
        rec["ok"] = ok
        rec["total_s"] = time.perf_counter() - t0
        out[name] = rec
    return out


# ---- the headline ---------------------------------------------------------------------------

def sustained(T, p, s, seconds, share):
    """The verify launch back to back for `seconds`, with the SM clock sampled meanwhile."""
    n, kernel_s, ops = 0, 0.0, 0
    with Clocks() as clk:
        t0 = time.perf_counter()
        while time.perf_counter() - t0 < seconds:
            r = T.enum_run(T.EN_VERIFY, p, spec=s, **share)
            assert r["hits"] == 0
            kernel_s += r["seconds"]
            ops += r["ops"]
            n += 1
        wall = time.perf_counter() - t0
    c = clk.summary() or {}
    rec = {"launches": n, "wall_s": wall, "kernel_s": kernel_s, "value": ops / kernel_s,
           "unit": "lane-ops/s", "ms_per_launch": 1e3 * kernel_s / n, "clocks": c or None}
    if c.get("sm_mhz"):
        # time x clock: cycles per launch, comparable across clocks
        rec["mcycles_per_launch"] = kernel_s / n * c["sm_mhz"]
    return rec


def headline(args):
    world, rank, local = dist_env()
    dist = None
    device = 0
    if world > 1:
        import torch.distributed as dist  # barrier and the result gather; no torch in the engine
        dist.init_process_group("gloo")
        if "CUDA_VISIBLE_DEVICES" not in os.environ:
            os.environ["CUDA_VISIBLE_DEVICES"] = str(local)  # this rank sees its GPU as 0
        elif len(os.environ["CUDA_VISIBLE_DEVICES"].split(",")) > local:
            device = local  # all GPUs visible: take this rank's

    import tesseract_gb300 as T
    from tesseract_gb300 import build, shard
    if rank == 0:
        build.build(reference=False)
    if dist:
        dist.barrier()
    err = T._err()
    if not T.lib().cuda_engine_init(device, err, len(err)):
        raise T.EngineError(err.value.decode())
    p = T.Program.gen_mul(16)
    s = T.Spec(p, "p = a * b")
    info = T.device_info()
    lop3 = T.lop3_peak()  # 32-bit LOP3 ops/s

    sharded = world > 1 and not args.replicas
    if sharded:
        part = dict(part=rank, part_end=rank, parts=world)
    else:
        part = dict(part=0, part_end=0, parts=args.share)
    tune = None
    if args.tune:  # the autotuner picks this job's kernel (block size, stretch) by measuring
        t0 = time.perf_counter()
        tune = T.enum_tune(T.EN_VERIFY, p, spec=s, **part)
        tune["seconds"] = time.perf_counter() - t0
    # untimed warm-up: at least W launches and at least half a second of them, so that the SM
    # clock, which drops while the host compiles and tunes, is at its level under load when the
    # timed region starts
    t_warm, n_warm = time.perf_counter(), 0
    while n_warm < max(3, args.warmup) or time.perf_counter() - t_warm < 0.5:
        r = T.enum_run(T.EN_VERIFY, p, spec=s, **part)
        assert r["hits"] == 0
        n_warm += 1
    stats = T.last_launch()

    if dist:
        dist.barrier()
    kernel_s, ops, tried, results = 0.0, 0, 0, []
    visible = os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")
    gpu = int(visible[min(device, len(visible) - 1)] or 0)
    with Clocks(gpu) as clk:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            r = T.enum_run(T.EN_VERIFY, p, spec=s, **part)
            kernel_s += r["seconds"]
            ops += r["ops"]
            tried += r["tried"]
            results.append(r)
        wall = time.perf_counter() - t0
    if dist:
        dist.barrier()
    assert all(x["hits"] == 0 for x in results), "verify found mismatches"
    merged = None
    if dist:
        import torch
        t = torch.tensor([wall, kernel_s], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        wall, kernel_s = float(t[0]), float(t[1])
        if sharded:  # the shares' records, gathered once and merged (src/work.c:341-371)
            merged = shard.gather_merge(results[-1])
        t = torch.tensor([ops, tried], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.SUM)
        ops, tried = int(t[0]), int(t[1])
    if rank != 0:
        return 0
    # a negative control outside the timed region: a wrong spec of the same shape must fail on
    # exactly the assignments where a != 0, so the kernel visibly checks every assignment
    control = None
    if args.share == 1:
        cs = T.Spec(p, "p = a * b + a")
        if sharded:
            cr = shard.merge([T.enum_run(T.EN_VERIFY, p, spec=cs, part=k, part_end=k,
                                         parts=world) for k in range(world)])
        else:
            cr = T.enum_run(T.EN_VERIFY, p, spec=cs)
        want = (1 << 32) - (1 << 16)
        control = {"spec": "p = a * b + a", "hits": cr["hits"], "expected": want,
                   "first_hits": cr["hit"][:4], "ok": cr["hits"] == want}
        assert control["ok"], control
    steps = args.steps
    value = ops / kernel_s          # kernel_s: the slowest rank's
    e2e = ops / wall
    launch_s = kernel_s / steps
    words = results[-1]["tried"] // 32            # per launch on one rank
    logic = stats["logic_ops_per_word"]
    achieved = logic * words / launch_s if logic else None
    lane_peak = lop3 * 32
    per_launch = results[-1]["ops"] / launch_s
    line = {
        "metric": METRIC, "value": value, "unit": "lane-ops/s", "n_gpus": world,
        "steps": steps, "warmup": args.warmup, "ms_per_step": 1e3 * launch_s,
        # the space is fixed and split into one share per rank (one share of the whole space at
        # N = 1); --replicas runs the whole space on every rank
        "higher_is_better": True, "scaling": "weak" if args.replicas else "strong",
        "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "assignments_per_s": tried / kernel_s,
        "config": {"workload": WORKLOAD + ("" if args.share == 1 else
                                           f" (share 0 of {args.share})"),
                   "assignments_per_step": tried // steps,
                   "lane_ops_per_step": ops // steps,
                   "l2": "no DRAM inputs: cell state lives in registers and every input word is "
                         "derived from the lane index, so there is nothing to flush",
                   "device": info,
                   "parallelism": (f"replicas x{world}" if args.replicas else
                                   f"--part shares x{world}")},
        "result": {"mismatches": 0, "tried_per_step": tried // steps,
                   "negative_control": control,
                   "merged_shares": ({k: merged[k] for k in ("space", "tried", "hits", "ops")}
                                     if merged else None)},
        "roofline": {
            "bound": "alu-lop3", "achieved": achieved, "peak": lop3, "unit": "LOP3/s",
            "frac": achieved / lop3 if achieved else None,
            "peak_source": "measured: cuda_lop3_peak microbenchmark on this GPU (32-bit LOP3/s)",
            "logic_ops_per_word": logic, "words_per_launch": words,
            "work_per_word": {"luts_per_step": stats["luts_per_step"],
                              "luts_per_stretch": stats["luts_per_stretch"],
                              "stretch_steps": stats["stretch_steps"],
                              "compare_ops": stats["compare_ops"]},
            "frac_accounting": per_launch / lane_peak,
            "accounting": {"achieved": per_launch, "peak": lane_peak, "unit": "lane-op/s",
                           "note": "the reference's 6,040 NAND/STO lane-ops per assignment "
                                   "over the LOP3 peak x 32 lanes"},
            "traffic": VERIFY_DRAM_BYTES if args.share == 1 and not sharded else None,
            "traffic_unit": "bytes per launch", "traffic_source": VERIFY_PROFILE,
            "alu_pipe_busy_ncu": VERIFY_ALU_PIPE_NCU},
        "kernel": {"regs": stats["regs"], "local_bytes": stats["local_bytes"],
                   "grid": stats["grid"], "block": stats["block"],
                   "compile_seconds": stats["compile_seconds"], "autotune": tune},
        "e2e": {"value": e2e, "unit": "lane-ops/s", "h2d_bytes_per_step": 72,
                "d2h_bytes_per_step": 8 + 4 * stats["grid"] * stats["block"] // 32,
                "path": "cuda_enum_run through the C ABI with host Program/Spec structs"},
        "gpu_launches": steps,
    }
    clocks = clk.summary()
    if clocks:
        line["clocks"] = clocks
    if args.sustained > 0:
        line["sustained"] = sustained(T, p, s, args.sustained, part)
    if args.configs and world == 1:
        line["configs"] = run_configs(args.configs.split(","))
    if not args.no_cpu:
        base, _, _ = cpu_sample()
        line["cpu_baseline"] = base
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--share", type=int, default=1,
                    help="verify only share 0 of this many (a small case for profiling)")
    ap.add_argument("--replicas", action="store_true",
                    help="N > 1: every rank verifies the whole space (default: --part shares)")
    ap.add_argument("--tune", type=int, default=1,
                    help="1: the autotuner picks the verify kernel before the warm-up")
    ap.add_argument("--sustained", type=float, default=5.0,
                    help="seconds of back-to-back launches after the timed steps (0: none)")
    ap.add_argument("--configs", default="life,batch,super,serve",
                    help="the other workloads run after the headline, comma separated ('' "
                         "for none)")
    ap.add_argument("--config", default="verify",
                    choices=["verify", "life", "batch", "super", "serve"],
                    help="one workload alone: verify is the headline line")
    ap.add_argument("--jobs", type=int, default=4096, help="batch: number of jobs")
    ap.add_argument("--gens", type=int, default=1000, help="life: generations")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.config != "verify":
        from tesseract_gb300 import build
        build.build(reference=False)
        if args.config == "life":
            rec, ok = config_life(args.gens)
        elif args.config == "batch":
            rec, ok = config_batch(args.jobs)
        elif args.config == "serve":
            rec, ok = config_serve(400 if args.jobs == 4096 else args.jobs)
        else:
            rec, ok = CONFIGS[args.config]()
        rec = dict(config=args.config, ok=ok, **rec)
        print(json.dumps(rec), flush=True)
        return 0 if ok else 3
    return headline(args)


if __name__ == "__main__":
    sys.exit(main())
