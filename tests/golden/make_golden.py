"""Regenerates the golden fixtures in this directory from the reference itself.

    python tests/golden/make_golden.py [path/to/alpha]          # programs.json, enum.json
    python tests/golden/make_golden.py --cli [path/to/alpha]    # cli.json
    python tests/golden/make_golden.py --tester1 [path/to/alpha]  # tester1.json
    python tests/golden/make_golden.py --cli-cpu [path/to/alpha]  # cli_cpu.json

Needs the reference's `alpha` binary built from its sources (oracle/Makefile builds it into
oracle/_ref/alpha on an x86 host that has the sources).  Programs come from the reference's own
generators (`alpha gen mul|hash`, `alpha random`) wherever it has one; the batched-equivalence
programs with inputs, which the reference cannot generate, come from this engine's generator and
are written out as assembly for the reference to read.  Every result is the reference's `--raw`
output (src/work.c:435-443): "EN mode space tried hits seconds threads ops" and "ENHIT x".

Outputs:
    programs.json   sha256 of the reference's generator output for each (kind, parameters)
    enum.json       enumeration cases and the reference's results
    cli.json        the reference's stdout and exit code for command lines of the hot path
    tester1.json    the reference's `tester1 --raw` histogram lines for a few configurations
    cli_cpu.json    the reference's stdout, stderr and exit code for command lines that need no
                    GPU: --merge of shares it wrote, option errors and refusals
"""
from __future__ import annotations

import hashlib
import json
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

ARGS = [a for a in sys.argv[1:] if not a.startswith("--")]
ALPHA = ARGS[0] if ARGS else os.path.join(ROOT, "oracle", "_ref", "alpha")


def run(args, stdin=None):
    r = subprocess.run([ALPHA] + args, capture_output=True, text=True)
    return r.returncode, r.stdout, r.stderr


def strip_comments(text):
    return "".join(l + "\n" for l in text.splitlines() if not l.startswith(";"))


def gen_text(kind, params):
    if kind == "mul":
        return strip_comments(run(["gen", "mul", "--bits", str(params["bits"])])[1])
    if kind == "hash":
        return strip_comments(run(["gen", "hash", "--bits", str(params["bits"]), "--rounds",
                                   str(params["rounds"])])[1])
    if kind == "life":
        return strip_comments(run(["gen", "life", "--size", str(params["size"])])[1])
    if kind == "random":
        return strip_comments(run(["random", "--cells", str(params["cells"]), "--len",
                                   str(params["len"]), "--seed", str(params["seed"])])[1])
    raise ValueError(kind)


def engine_text(kind, params):
    """Programs the reference cannot generate: this engine's generator, as assembly."""
    import tesseract_gb300 as T
    if kind == "random_in":
        p = T.Program.random_in(params["cells"], params["width"], params["len"], params["seed"])
    elif kind == "rewrite":
        base = T.Program.random_in(params["cells"], params["width"], params["len"],
                                   params["seed"])
        p = base.rewrite(params["rseed"], params.get("mutate", False))
    else:
        raise ValueError(kind)
    return p.text()


def parse_raw(out):
    res = {"hit": []}
    for line in out.splitlines():
        f = line.split()
        if f and f[0] == "EN":
            res.update(mode=int(f[1]), space=int(f[2]), tried=int(f[3]), hits=int(f[4]),
                       ops=int(f[7]))
        elif f and f[0] == "ENHIT":
            res["hit"].append(int(f[1], 16))
    return res


def program_file(tmp, prog):
    kind, params = prog["kind"], prog["params"]
    text = engine_text(kind, params) if kind in ("random_in", "rewrite") else gen_text(kind, params)
    path = os.path.join(tmp, hashlib.sha1(json.dumps(prog, sort_keys=True).encode()).hexdigest()
                        + ".asm")
    with open(path, "w") as f:
        f.write(text)
    return path


def cases():
    mul = lambda b: {"kind": "mul", "params": {"bits": b}}
    out = []
    for b in range(1, 9):
        out.append({"mode": "verify", "a": mul(b), "spec": "p = a * b"})
    for spec in ["p = a * b + 1", "p = a + b", "p = (a * b) >> 1", "p = a * b - (a << 2)",
                 "p = ~a & b | 3", "p = -a ^ b", "p = a * b >> 64", "p = a * b << 65",
                 "p = (a * b) ^ (b << 3)", "p = a * 3 + b * 5 - 7", "p = a & b ^ a | b",
                 "p = a << b", "p = (a * b) >> (b & 7)"]:
        out.append({"mode": "verify", "a": mul(6), "spec": spec})
    # a left side wider than 32 bits: 20 x 20 -> 40-bit product, one share of 65536
    out.append({"mode": "verify", "a": mul(20), "spec": "p = a * b", "part": [0, 0, 65536]})
    out.append({"mode": "verify", "a": mul(20), "spec": "p = a * b + 0x100000000",
                "part": [3, 3, 65536]})
    out.append({"mode": "verify", "a": mul(18), "spec": "p = a * b ^ (a << 30)",
                "part": [7, 9, 16384]})
    # shares, as on the cluster (tests/test_work.c:269-290)
    for part in ([0, 0, 3], [1, 1, 3], [2, 2, 3], [0, 1, 3], [5, 6, 7]):
        out.append({"mode": "verify", "a": mul(10), "spec": "p = a * b ^ 1", "part": part})
    # ticks > 1 on a combinational program: the same answer
    out.append({"mode": "verify", "a": mul(5), "spec": "p = a * b", "ticks": 3})
    # specs that are a sum of a part without the fastest-changing inputs and a part without the
    # lane inputs, on multipliers whose enumeration order the engine permutes
    for spec in ["p = a * b + a", "p = a * b * 3 - b", "p = a * b << 3"]:
        out.append({"mode": "verify", "a": mul(12), "spec": spec})
    out.append({"mode": "verify", "a": mul(16), "spec": "p = a * b + a", "part": [5, 5, 4096]})
    out.append({"mode": "verify", "a": mul(16), "spec": "p = a * b", "part": [0, 1, 4096]})
    # search: toy hash preimages (tests/test_work.c:322-376)
    for bits, rounds, x in ((3, 5, 5), (16, 5, 12345), (20, 8, 777), (24, 8, 0xabcdef)):
        out.append({"mode": "search", "a": {"kind": "hash", "params": {"bits": bits,
                                                                         "rounds": rounds}},
                    "want_x": x, "bits": bits, "rounds": rounds})
    # equiv: random programs with inputs against rewritten copies, and mutated controls
    for seed, (cells, width, length) in enumerate([(8, 5, 40), (16, 12, 300), (24, 16, 900),
                                                   (9, 20, 200), (40, 18, 2000), (64, 22, 4096),
                                                   (12, 3, 50), (30, 14, 1500)]):
        base = {"cells": cells, "width": width, "len": length, "seed": 1000 + seed}
        a = {"kind": "random_in", "params": base}
        for mutate in (False, True):
            b = {"kind": "rewrite", "params": dict(base, rseed=77 + seed, mutate=mutate)}
            out.append({"mode": "equiv", "a": a, "b": b})
    out.append({"mode": "equiv", "a": {"kind": "random_in", "params": {"cells": 10, "width": 9,
                                                                       "len": 120, "seed": 5}},
                "b": {"kind": "rewrite", "params": {"cells": 10, "width": 9, "len": 120,
                                                    "seed": 5, "rseed": 6, "mutate": True}},
                "ticks": 4})
    return out


def main():
    import tesseract_gb300 as T
    from tesseract_gb300 import build
    build.build(reference=False)
    progs = {}
    for kind, plist in (("mul", [{"bits": b} for b in (1, 2, 3, 4, 5, 6, 7, 8, 10, 12, 16, 18,
                                                       20)]),
                        ("hash", [{"bits": b, "rounds": r} for b, r in ((3, 5), (16, 5), (20, 8),
                                                                        (24, 8), (32, 8),
                                                                        (40, 8))]),
                        ("life", [{"size": s} for s in (3, 8, 10, 32)]),
                        ("random", [{"cells": c, "len": l, "seed": s}
                                    for c, l, s in ((8, 20, 3), (64, 4096, 1), (100, 1000, 42))])):
        for params in plist:
            key = kind + ":" + json.dumps(params, sort_keys=True)
            progs[key] = hashlib.sha256(gen_text(kind, params).encode()).hexdigest()
    with open(os.path.join(HERE, "programs.json"), "w") as f:
        json.dump(progs, f, indent=1, sort_keys=True)

    results = []
    with tempfile.TemporaryDirectory() as tmp:
        for c in cases():
            pa = program_file(tmp, c["a"])
            args = [c["mode"], pa]
            if c["mode"] == "equiv":
                args.append(program_file(tmp, c["b"]))
            if c["mode"] == "verify":
                args += ["--spec", c["spec"]]
            if c["mode"] == "search":
                target = T.lib().tc_toyhash(c["want_x"] % (1 << c["bits"]), c["bits"],
                                            c["rounds"])
                c["spec"] = "h = %d" % target
                args += ["--want", c["spec"]]
            if "ticks" in c:
                args += ["--ticks", str(c["ticks"])]
            if "part" in c:
                i, j, k = c["part"]
                args += ["--part", "%d-%d/%d" % (i, j, k)]
            args += ["--raw"]
            rc, out, errtext = run(args)
            if rc != 0:
                raise RuntimeError(" ".join(args) + ": " + errtext)
            c["result"] = parse_raw(out)
            results.append(c)
            print(c["mode"], c["a"]["kind"], c.get("spec", ""), c["result"]["hits"], flush=True)
    with open(os.path.join(HERE, "enum.json"), "w") as f:
        json.dump(results, f, indent=1)


if __name__ == "__main__" and not {"--cli", "--tester1", "--cli-cpu"} & set(sys.argv):
    main()


# ---- the command line: the reference's stdout for the same commands -------------------------

CLI_CASES = [
    (["verify", "{mul4}", "--spec", "p = a * b"], None),
    (["verify", "{mul4}", "--spec", "p = a * b + 1"], None),
    (["verify", "{mul6}", "--spec", "p = a * b ^ 1", "--part", "0/3"], None),
    (["verify", "{mul6}", "--spec", "p = a * b ^ (a >> 2)", "--raw"], None),
    (["equiv", "{ra}", "{rb}"], None),
    (["equiv", "{ra}", "{rc}"], None),
    (["search", "{hash16}", "--want", "h = 34272"], None),
    (["search", "{hash16}", "--want", "h = 34272", "--raw"], None),
    (["verify", "{mul5}", "--spec", "p = a * b", "--ticks", "2"], None),
    # run --table (src/main.c:422-445): the truth table, .out columns or RR
    (["run", "{mul3}", "--table"], None),
    (["run", "{rt}", "--table"], None),
    (["run", "{rt}", "--table", "--ticks", "3"], None),
    (["run", "{rr}", "--table", "--ticks", "2"], None),
    # check (src/main.c:503-567), life (src/work.c:490-701), cube (src/cubedemo.c:549-623),
    # super (src/supercmd.c:81-180), tester1 --raw (src/main.c:1071-1160): the kind names how
    # tests/test_cli_gpu.py compares them (timings, engine names and search traces aside)
    (["check", "{mul4}"], "check"),
    (["check", "{rt}", "--ticks", "3", "--seed", "7"], "check"),
    (["check", "{links10}"], "check"),
    (["life", "--gens", "5", "--size", "8", "--show", "--seconds", "0"], "life"),
    (["life", "--gens", "7", "--seconds", "0"], "life"),
    (["life", "--cube", "--size", "8", "--gens", "4", "--seconds", "0"], "life"),
    (["life", "--dims", "10", "--size", "8", "--gens", "3", "--show", "--seconds", "0"], "life"),
    (["life", "--dims", "11", "--rows", "3", "--size", "4", "--gens", "5", "--seconds", "0"],
     "life"),
    (["life", "--size", "2"], "life"),
    (["cube", "--checks", "3", "--seconds", "0.01"], "cube"),
    (["cube", "any", "--dims", "10", "--seconds", "0.01"], "cube"),
    (["cube", "rank", "--dims", "10", "--seconds", "0.01"], "cube"),
    (["cube", "sort", "--dims", "10", "--seconds", "0.01"], "cube"),
    (["super", "RR = RR ^ x"], "super"),
    (["super", "o{{x,y}} = x ^ y"], "super"),
    (["super", "r{{a,b}} = s ? a : b"], "super"),
    (["tester1", "--programs", "8", "--raw", "--threads", "1"], "tester1"),
]

RR_ONLY = ".in x y z\nNAND x\nNAND y\nSTO t\nNAND z\nNAND t\nSTO x\n"



def cli_programs(tmp):
    import tesseract_gb300 as T
    progs = {}
    for name, text in (("mul4", gen_text("mul", {"bits": 4})), ("mul5", gen_text("mul", {"bits": 5})),
                       ("mul6", gen_text("mul", {"bits": 6})),
                       ("hash16", gen_text("hash", {"bits": 16, "rounds": 5}))):
        progs[name] = text
    a = T.Program.random_in(12, 10, 200, 424242)
    progs["ra"] = a.text()
    progs["rb"] = a.rewrite(5).text()
    progs["rc"] = a.rewrite(5, mutate=True).text()
    progs["mul3"] = gen_text("mul", {"bits": 3})
    progs["rt"] = T.Program.random_in(6, 5, 40, 7).text()
    progs["rr"] = RR_ONLY
    progs["links10"] = (".in x\n.out y z\n.link l = x @ 9\n.link k = l @ 2\nNAND l\nSTO y\n"
                        "NAND k\nNAND ID3\nSTO z\nNAND ID9\nSTO x\n")
    paths = {}
    for k, v in progs.items():
        paths[k] = os.path.join(tmp, k + ".asm")
        with open(paths[k], "w") as f:
            f.write(v)
    return progs, paths


def cli_main():
    global ALPHA
    out = []
    with tempfile.TemporaryDirectory() as tmp:
        progs, paths = cli_programs(tmp)
        # the cube demos read lib/std.inc beside the binary's directory: a copy of the binary
        # in tmp/bin next to a link to the reference's lib
        import shutil
        os.makedirs(os.path.join(tmp, "bin"))
        shutil.copy(ALPHA, os.path.join(tmp, "bin", "alpha"))
        with open(os.path.join(ROOT, "oracle", "_ref", "SOURCE")) as f:
            os.symlink(os.path.join(f.read().strip(), "lib"), os.path.join(tmp, "lib"))
        ALPHA = os.path.join(tmp, "bin", "alpha")
        for args, kind in CLI_CASES:
            real = [a.format(**paths) for a in args]
            rc, stdout, stderr = run(real)
            text = stdout.replace(tmp + "/", "")
            out.append({"args": args, "rc": rc, "stdout": text, "kind": kind or "enum"})
    with open(os.path.join(HERE, "cli.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__" and "--cli" in sys.argv:
    cli_main()


# ---- tester1: the reference's raw histogram lines (one thread, so the order is fixed) --------

T1_CASES = [
    ["--programs", "16"],
    ["--cells", "8,100,500,1000", "--programs", "8", "--max-passes", "4096", "--seed", "7"],
    ["--cells", "20,40", "--ratio", "2", "--programs", "32", "--max-passes", "64"],
    ["--cells", "3,5", "--ratio", "9", "--programs", "40", "--seed", "12345"],
]


def t1_main():
    out = []
    for args in T1_CASES:
        rc, stdout, stderr = run(["tester1"] + args + ["--raw", "--threads", "1"])
        if rc != 0:
            raise RuntimeError(stderr)
        lines = [l for l in stdout.splitlines() if l.startswith("T1 ")]
        out.append({"args": args, "t1": lines})
    with open(os.path.join(HERE, "tester1.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__" and "--tester1" in sys.argv:
    t1_main()


# ---- the command line without a GPU: merged shares, option errors, refusals -------------------

# (args, shares): shares are command lines whose --raw output the reference writes into the files
# {raw0}, {raw1}, ... named by args; every other case runs as given.
CLI_CPU_CASES = [
    (["verify", "{mul10}", "--spec", "p = a * b ^ (a & 1)", "--merge", "{raw0}", "{raw1}",
      "{raw2}"],
     [["verify", "{mul10}", "--spec", "p = a * b ^ (a & 1)", "--part", f"{i}/3", "--raw"]
      for i in range(3)]),
    (["verify", "{mul10}", "--spec", "p = a * b ^ (a & 1)", "--merge", "{raw0}", "{raw1}"],
     [["verify", "{mul10}", "--spec", "p = a * b ^ (a & 1)", "--part", "0-1/4", "--raw"],
      ["verify", "{mul10}", "--spec", "p = a * b ^ (a & 1)", "--part", "3/4", "--raw"]]),
    (["verify", "{mul10}", "--spec", "p = a * b", "--merge", "{raw0}", "{raw1}"],
     [["verify", "{mul10}", "--spec", "p = a * b", "--part", f"{i}/2", "--raw"]
      for i in range(2)]),
    (["equiv", "{ra}", "{rc}", "--merge", "{raw0}", "{raw1}"],
     [["equiv", "{ra}", "{rc}", "--part", f"{i}/2", "--raw"] for i in range(2)]),
    (["search", "{hash16}", "--want", "h = 34272", "--merge", "{raw0}", "{raw1}"],
     [["search", "{hash16}", "--want", "h = 34272", "--part", f"{i}/2", "--raw"]
      for i in range(2)]),
    (["search", "{hash16}", "--want", "h = 1", "--merge", "{raw0}"],
     [["search", "{hash16}", "--want", "h = 1", "--part", "0/1", "--raw"]]),
    (["verify", "{mul10}", "--spec", "p = a * b", "--merge", "{raw0}", "missing.raw"],
     [["verify", "{mul10}", "--spec", "p = a * b", "--part", "0/2", "--raw"]]),
    # tester1 --merge (src/tester.c:279-429): shares of several sizes, a passes limit that
    # leaves runs without a cycle, a time limit that cuts programs off, a missing file
    (["tester1", "--merge", "{raw0}", "{raw1}"],
     [["tester1", "--cells", "8,16,32", "--programs", "8", "--raw", "--threads", "1"],
      ["tester1", "--cells", "16,64", "--programs", "6", "--seed", "9", "--raw", "--threads",
       "2"]]),
    (["tester1", "--merge", "{raw0}", "{raw1}"],
     [["tester1", "--cells", "100,400", "--programs", "6", "--max-passes", "256", "--raw",
       "--threads", "1"],
      ["tester1", "--cells", "3000", "--ratio", "8", "--seconds", "0.3", "--raw", "--threads",
       "2"]]),
    (["tester1", "--programs", "2", "--merge", "{raw0}", "missing.raw"],
     [["tester1", "--cells", "8", "--programs", "2", "--raw", "--threads", "1"]]),
    (["verify"], []),
    (["verify", "{mul4}"], []),
    (["search", "{mul4}"], []),
    (["verify", "{mul4}", "--spec"], []),
    (["verify", "{mul4}", "--spec", "p = a * b", "--ticks", "0"], []),
    (["verify", "{mul4}", "--spec", "p = a * b", "--ticks", "x"], []),
    (["verify", "{mul4}", "--spec", "p = a * b", "--ticks"], []),
    (["verify", "{mul4}", "--spec", "p = a * b", "--part", "1"], []),
    (["verify", "{mul4}", "--spec", "p = a * b", "--part", "1-x/4"], []),
    (["verify", "{mul4}", "--spec", "p = a * b", "--bogus"], []),
    (["verify", "{mul4}", "--spec", "q = a"], []),
    (["verify", "{mul4}", "--spec", "p = a +"], []),
    (["search", "{hash16}", "--want", "h = x"], []),
    (["verify", "missing.asm", "--spec", "p = a"], []),
    (["equiv", "{ra}", "{mul4}"], []),
    (["equiv", "{mul4}", "missing.asm"], []),
    (["verify", "{links}", "--spec", "y = x"], []),
    (["verify", "{mul4}", "--spec", "p = a * b", "--part", "3/2"], []),
]


def cli_cpu_main():
    out = []
    with tempfile.TemporaryDirectory() as tmp:
        progs, paths = cli_programs(tmp)
        extra = {"mul10": gen_text("mul", {"bits": 10}),
                 "links": ".in x\n.out y\n.link l = x @ 3\nNAND l\nSTO y\n"}
        for k, v in extra.items():
            paths[k] = os.path.join(tmp, k + ".asm")
            with open(paths[k], "w") as f:
                f.write(v)
        for args, shares in CLI_CPU_CASES:
            raws = []
            for i, sh in enumerate(shares):
                rc, stdout, stderr = run([a.format(**paths) for a in sh])
                assert rc == 0, (sh, stderr)
                raws.append(stdout)
                paths["raw%d" % i] = os.path.join(tmp, "raw%d" % i)
                with open(paths["raw%d" % i], "w") as f:
                    f.write(stdout)
            cwd = os.getcwd()
            os.chdir(tmp)
            try:
                rc, stdout, stderr = run([a.format(**paths) for a in args])
            finally:
                os.chdir(cwd)
            out.append({"args": args, "raws": raws, "rc": rc,
                        "stdout": stdout.replace(tmp + "/", ""),
                        "stderr": stderr.replace(tmp + "/", "")})
    with open(os.path.join(HERE, "cli_cpu.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__" and "--cli-cpu" in sys.argv:
    cli_cpu_main()
