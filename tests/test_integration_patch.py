"""The patch INTEGRATION.md describes (tests/integration/engine_cuda.patch: `--engine cuda` in
verify/equiv/search, check and run --table, and the GPU superoptimizer) applied to a copy of the
reference's own sources: the patched files compile against the reference's headers with
include/tesseract_cuda.h after them, the patched reference links against this engine's library
without a clashing symbol, and runs its CPU engines as before.  Needs the reference's sources
(recorded by oracle/Makefile) and an x86 host (its lane engine is AVX2)."""
import os
import platform
import shutil
import subprocess

import pytest

import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PATCH = os.path.join(ROOT, "tests", "integration", "engine_cuda.patch")
LIBDIR = os.path.join(ROOT, "tesseract_gb300")
SRC = O.reference_sources()

pytestmark = pytest.mark.skipif(not SRC or platform.machine() not in ("x86_64", "AMD64"),
                                reason="needs the reference's sources on an x86 host")


@pytest.fixture(scope="module")
def patched(tmp_path_factory):
    d = tmp_path_factory.mktemp("ref")
    shutil.copytree(os.path.join(SRC, "src"), d / "src")
    shutil.copytree(os.path.join(SRC, "lib"), d / "lib")
    for f in (d / "src").iterdir():
        f.chmod(0o644)
    r = subprocess.run(["patch", "-p1", "-i", PATCH], cwd=d, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return d


def test_patched_files_compile_against_the_reference_headers(patched):
    for f in ("work.c", "main.c", "supercmd.c"):
        r = subprocess.run(["gcc", "-std=c11", "-D_GNU_SOURCE", "-fsyntax-only", "-Wall",
                            "-Werror", "-I.", "-I" + os.path.join(ROOT, "include"), f],
                           cwd=patched / "src", capture_output=True, text=True)
        assert r.returncode == 0, f + ": " + r.stderr


def test_patched_reference_links_and_runs(patched):
    src = patched / "src"
    srcs = sorted(str(p.name) for p in src.iterdir() if p.suffix == ".c" and p.name != "lanes.c")
    (patched / "bin").mkdir()
    cmd = ["gcc", "-std=c11", "-O1", "-D_GNU_SOURCE", "-w", "-I.",
           "-I" + os.path.join(ROOT, "include"), "-mavx2", "lanes.c"] + srcs + \
          ["-o", str(patched / "bin" / "alpha"), "-pthread", "-L" + LIBDIR, "-ltesseract_gb300",
           "-Wl,-rpath," + LIBDIR, "-lm"]
    r = subprocess.run(cmd, cwd=src, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    alpha = str(patched / "bin" / "alpha")
    gen = subprocess.run([alpha, "gen", "mul", "--bits", "5"], capture_output=True, text=True)
    (patched / "m5.asm").write_text(gen.stdout)
    r = subprocess.run([alpha, "verify", "m5.asm", "--spec", "p = a * b"], cwd=patched,
                       capture_output=True, text=True)
    assert r.returncode == 0 and "OK: the outputs equal the spec" in r.stdout, r.stderr
    r = subprocess.run([alpha, "check", "m5.asm", "--engine", "jit"], cwd=patched,
                       capture_output=True, text=True)
    assert r.returncode == 0 and "OK: the compiled code matches" in r.stdout
    # --engine cuda reaches this engine: on a host without a GPU it reports that, not a crash
    r = subprocess.run([alpha, "verify", "m5.asm", "--spec", "p = a * b", "--engine", "cuda"],
                       cwd=patched, capture_output=True, text=True, timeout=120)
    assert r.returncode in (0, 1), r.stderr
    assert r.returncode == 0 or "CUDA" in r.stderr or "device" in r.stderr, r.stderr
