"""Builds the native parts in-tree: ``lassie_gb300/_native/liblassie_gb300.so``
(sm_103a kernels + C ABI) and the ``lassie`` CLI binary.

Translation units compile in parallel; nothing here needs cmake.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from typing import List

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_native")
INCLUDE = os.path.join(ROOT, "include")
LIB = os.path.join(OUT, "liblassie_gb300.so")
CLI = os.path.join(OUT, "lassie")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# --fmad=false: no implicit a*b+c contraction; fused operations in the
# engine are written as explicit fma, matching the CPU oracle.
NVCC_FLAGS = ["-std=c++17", "-O3", "--fmad=false", "-lineinfo", "-Xcompiler", "-fPIC",
              "-I" + INCLUDE, "-I" + CSRC] + ARCH

SOURCES = ["compat_engine.cu", "capi.cu", "noalloc.cu", "float_mode.cu"]
# The reference's single-precision mode is compiled with the reference's own
# device flags (fast float division, pow and sqrt, flush-to-zero, FMA
# contraction), so that its float expressions round as the reference's do.
FILE_FLAGS = {"float_mode.cu": ["-std=c++17", "-O3", "--use_fast_math", "-lineinfo", "-Xcompiler",
                                "-fPIC", "-I" + INCLUDE, "-I" + CSRC] + ARCH}


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: List[str]) -> None:
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout)


def _stale(target: str, deps: List[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile the kernels, the C ABI library and the CLI.  Returns the
    library path."""
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(INCLUDE, "lassie_gb300.h"))
    objs, jobs = [], []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc] + FILE_FLAGS.get(src, NVCC_FLAGS) + ["-c", s, "-o", o])
    if jobs:
        with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            for _ in ex.map(_run, jobs):
                pass
    if force or jobs or _stale(LIB, objs):
        _run([nvcc, "-shared", "-o", LIB] + objs + ARCH + ["-Xcompiler", "-fPIC"])
    cli_src = os.path.join(HERE, "cli", "lassie_main.cpp")
    if force or _stale(CLI, [cli_src, LIB, os.path.join(INCLUDE, "lassie_gb300.h")]):
        gxx = shutil.which("g++") or "g++"
        _run([gxx, "-std=c++17", "-O2", "-I" + INCLUDE, cli_src, "-o", CLI, "-L" + OUT,
              "-llassie_gb300", "-Wl,-rpath,$ORIGIN"])
    if verbose:
        print("built", LIB, CLI, file=sys.stderr)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
