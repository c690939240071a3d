"""Builds the engine library libqgpu.so for sm_103a (GB300) in-tree.

The translation units are compiled in parallel with nvcc and linked into
``qsource_gb300/_build/libqgpu.so``; nothing is installed.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
SOURCES = ["qgpu_api.cu", "k_lists.cu", "k_pairs.cu", "k_small.cu", "k_md.cu", "k_lrf_static.cu", "qgpu_ene.cu", "k_mlp.cu",
           "qgpu_calc.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I" + os.path.join(ROOT, "include"),
         "-I" + CSRC, "--use_fast_math=false"]
# The FP32 pair and list kernels never meet subnormal values (distances of
# 0.5-100 A, charges and LJ products far from 1e-38): flush-to-zero lets
# rsqrtf and the FP32 arithmetic skip subnormal handling (3-4 % faster).
# Division and square root stay IEEE-rounded.
FILE_FLAGS = {"k_pairs.cu": ["-ftz=true"], "k_lists.cu": ["-ftz=true"]}


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _up_to_date(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def build(verbose: bool = False, force: bool = False, extra: list[str] | None = None) -> str:
    """Compile every CUDA translation unit and link libqgpu.so; returns its path."""
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith(".cuh")]
    headers.append(os.path.join(ROOT, "include", "qgpu.h"))
    flags = FLAGS[:-1] + (extra or [])
    objs = []
    jobs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src.replace(".cu", ".o"))
        objs.append(o)
        if force or not _up_to_date(o, [s] + headers):
            jobs.append([nvcc, *ARCH, *flags, *FILE_FLAGS.get(src, []), "-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        for cmd, res in zip(jobs, ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs)):
            if verbose or res.returncode:
                sys.stderr.write(res.stdout + res.stderr)
            if res.returncode:
                raise RuntimeError("nvcc failed: " + " ".join(cmd))
    lib = os.path.join(OUT, "libqgpu.so")
    if force or jobs or not _up_to_date(lib, objs):
        res = subprocess.run([nvcc, *ARCH, "-shared", "-o", lib, *objs, "-lcudart"], capture_output=True, text=True)
        if res.returncode:
            sys.stderr.write(res.stdout + res.stderr)
            raise RuntimeError("link failed")
    return lib


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
