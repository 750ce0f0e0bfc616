"""Compile the CUDA pipeline into _build/libpfcuda.so (sm_103a only).

Each translation unit is compiled in its own nvcc process, in parallel, then linked.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libpfcuda.so")
NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code without FMA contraction: the SVG parser and the host-side arithmetic follow the
# reference operation by operation on x86 and on Arm
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off", "-I", os.path.join(ROOT, "include")]


def sources():
    return sorted(glob.glob(os.path.join(HERE, "csrc", "*.cu")))


def _newer(target: str, deps) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def build(verbose: bool = False, extra=None) -> str:
    os.makedirs(OUT, exist_ok=True)
    headers = glob.glob(os.path.join(HERE, "csrc", "*.h")) + glob.glob(os.path.join(ROOT, "include", "*.h"))
    srcs = sources()
    objs = [os.path.join(OUT, os.path.basename(s)[:-3] + ".o") for s in srcs]
    extra = list(extra or [])

    def one(src_obj):
        src, obj = src_obj
        if _newer(obj, [src] + headers):
            return ""
        cmd = [NVCC] + ARCH + FLAGS + extra + ["-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        return r.stderr

    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        for msg in ex.map(one, zip(srcs, objs)):
            if verbose and msg:
                print(msg, file=sys.stderr)
    if not _newer(LIB, objs):
        cmd = [NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, extra=sys.argv[1:]))
