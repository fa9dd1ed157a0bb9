"""Builds the engine's shared library, its command line tool and the oracle, in place.

    python -m tesseract_gb300.build [-v]

Products (all git-ignored, rebuilt on each machine):
    tesseract_gb300/libtesseract_gb300.so   the C ABI (include/tesseract_cuda.h): host C + CUDA
    tesseract_gb300/bin/alpha-cuda          the reference's command line over the CUDA engine
    oracle/liboracle.so                     the CPU oracle (test infrastructure)
    oracle/_ref/{alpha,libalpha.so}         the reference itself, only where its sources exist

Host C is compiled with gcc (C11), CUDA sources with nvcc for sm_103a only
(-gencode arch=compute_103a,code=sm_103a); the generated per-program kernels are compiled at
run time by NVRTC for the device's own architecture.  Objects whose sources and headers are
older than the object are not rebuilt.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "tesseract_gb300")
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(ROOT, "_build")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# The reference's source tree, for oracle/_ref (golden fixtures and the x86 CPU baseline only).
# This build recipe is the one place that names where it is mounted; TESSERACT_REFERENCE
# overrides it, and the step is skipped where the tree is absent (the GPU machine).
REFERENCE = os.environ.get("TESSERACT_REFERENCE", "/root/reference")

HOST_C = ["program", "asm", "spec", "gen", "lutmap", "codegen", "ptxgen", "engine", "cube", "ref_host", "batch", "tester",
          "serve", "super_host", "cli_support"]
CUDA_SRC = ["peak_kernels", "batch_kernels", "super_kernels", "enum_static", "tester_kernels"]
CFLAGS = ["-std=c11", "-O2", "-g", "-Wall", "-Wextra", "-fPIC", "-D_GNU_SOURCE",
          "-I" + os.path.join(CUDA, "include")]
NVFLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                  "-I" + os.path.join(CUDA, "include")]

LIB = os.path.join(PKG, "libtesseract_gb300.so")
CLI = os.path.join(PKG, "bin", "alpha-cuda")
ORACLE_LIB = os.path.join(ROOT, "oracle", "liboracle.so")


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs += [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    return hs


def _stale(out, inputs):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(i) > t for i in inputs if os.path.exists(i))


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build(verbose: bool = False, reference: bool = True) -> dict:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(os.path.dirname(CLI), exist_ok=True)
    headers = _headers()
    jobs = []
    objs = []
    for name in HOST_C:
        src = os.path.join(CSRC, name + ".c")
        if not os.path.exists(src):
            continue
        obj = os.path.join(BUILD, name + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            jobs.append(["gcc"] + CFLAGS + ["-c", src, "-o", obj])
    for name in CUDA_SRC:
        src = os.path.join(CSRC, name + ".cu")
        if not os.path.exists(src):
            continue
        obj = os.path.join(BUILD, name + ".cu.o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            jobs.append([NVCC] + NVFLAGS + ["-c", src, "-o", obj])
    oracle_src = os.path.join(ROOT, "oracle", "oracle.c")
    oracle_jobs = []
    if _stale(ORACLE_LIB, [oracle_src] + headers):
        oracle_jobs.append(["gcc", "-std=c11", "-O2", "-g", "-fPIC", "-shared", "-pthread",
                            "-D_GNU_SOURCE", "-Wall", oracle_src, "-o", ORACLE_LIB])
    with cf.ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        list(ex.map(lambda c: _run(c, verbose), jobs + oracle_jobs))
    cuda_lib = os.path.join(CUDA, "lib64")
    if _stale(LIB, objs):
        _run([NVCC] + ARCH + ["-shared", "-o", LIB] + objs +
             ["-L" + cuda_lib, "-lnvrtc", "-lnvJitLink", "-Xlinker", "-rpath," + cuda_lib, "-lpthread"], verbose)
    cli_src = os.path.join(CSRC, "cli.c")
    if os.path.exists(cli_src) and _stale(CLI, [cli_src, LIB] + headers):
        _run(["gcc"] + CFLAGS + [cli_src, "-o", CLI, "-L" + PKG, "-ltesseract_gb300",
                                 "-Wl,-rpath,$ORIGIN/..", "-lm"], verbose)
    out = {"lib": LIB, "cli": CLI if os.path.exists(CLI) else None, "oracle": ORACLE_LIB}
    if reference and os.path.isdir(os.path.join(REFERENCE, "src")) and shutil.which("make"):
        # the reference's own binary and library, from its sources (x86 only: AVX2 lane engine)
        import platform
        if platform.machine() in ("x86_64", "AMD64"):
            _run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "-j8", "REF=" + REFERENCE],
                 verbose)
            out["reference"] = os.path.join(ROOT, "oracle", "_ref", "alpha")
    return out


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
