"""Build recipe of the sm_103a library, the fz-gpu CLI and the oracle.

    python fz-gpu_gb300/build.py            # library + CLI (in-tree, parallel nvcc)

Outputs (git-ignored): fz-gpu_gb300/_build/*.o, fz-gpu_gb300/libfzgb300.so,
fz-gpu_gb300/fz-gpu.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libfzgb300.so")
CLI = os.path.join(HERE, "fz-gpu")

CU_SOURCES = ["fz_compress.cu", "fz_decompress.cu", "fz_api.cu", "fz_noalloc.cu", "fz_server.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xptxas", "-O3",
              "--expt-relaxed-constexpr", "-I" + os.path.join(ROOT, "include")]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def cuda_home() -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc())))


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(ROOT, "include", "fz.h"))
    return hs


def compile_one(src: str, verbose=False) -> str:
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    s = os.path.join(CSRC, src)
    if _stale(obj, [s] + _headers()):
        cmd = [nvcc()] + ARCH + NVCC_FLAGS + ["-c", s, "-o", obj]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        if verbose:
            sys.stderr.write(r.stderr)
    return obj


def build(verbose=False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(CU_SOURCES)) as ex:
        objs = list(ex.map(lambda s: compile_one(s, verbose), CU_SOURCES))
    if _stale(LIB, objs):
        subprocess.check_call([nvcc()] + ARCH + ["-shared", "-o", LIB] + objs +
                              ["-lcudart"])
    cli_src = os.path.join(CSRC, "fz_cli.cpp")
    if _stale(CLI, [cli_src, LIB, os.path.join(ROOT, "include", "fz.h")]):
        home = cuda_home()
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "include"),
                               "-I" + os.path.join(home, "include"), cli_src, "-o", CLI,
                               "-L" + HERE, "-lfzgb300", "-L" + os.path.join(home, "lib64"),
                               "-lcudart", "-Wl,-rpath,$ORIGIN", "-Wl,-rpath," + os.path.join(home, "lib64")])
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
