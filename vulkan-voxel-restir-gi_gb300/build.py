"""Build recipe of the native library (libvrg.so) for sm_103a.

Every translation unit is compiled by nvcc in parallel and linked into one
shared library next to this file.  Numerics flags are part of the contract:
-fmad=false (no FMA contraction on the device), IEEE division and square root,
no flush-to-zero, and -ffp-contract=off for host code, so that the device
computes each float expression as the same sequence of binary32 operations a
host compiler produces.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libvrg.so")

SOURCES = ["api.cpp", "terrain.cpp", "image.cpp", "sah.cu", "extract.cu", "scene.cu", "trace.cu", "restir.cu", "nrc.cu", "peaks.cu", "mesh.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17",
    "-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false",
    "-Xcompiler", "-fPIC,-ffp-contract=off,-fvisibility=hidden,-O2",
    "-I", os.path.join(HERE, "..", "include"),
]


def nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def _compile(src, extra):
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), "-c", os.path.join(CSRC, src), "-o", obj] + NVCC_FLAGS + extra
    r = subprocess.run(cmd, capture_output=True, text=True)
    return src, obj, r


def build(verbose=False, extra=()):
    os.makedirs(BUILD, exist_ok=True)
    extra = list(extra)
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(lambda s: _compile(s, extra), SOURCES))
    failed = [(s, r) for s, _, r in results if r.returncode != 0]
    for s, _, r in results:
        if verbose and (r.stdout or r.stderr):
            sys.stderr.write(f"--- {s}\n{r.stdout}{r.stderr}")
    if failed:
        msg = "\n".join(f"--- {s}\n{r.stdout}{r.stderr}" for s, r in failed)
        raise RuntimeError("nvcc failed:\n" + msg)
    objs = [o for _, o, _ in results]
    tmp = LIB + ".tmp"
    cmd = [nvcc(), "-shared", "-o", tmp] + objs + ARCH + ["-lcudart_static", "-lrt", "-ldl", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, extra=["-Xptxas", "-v"] if "--ptxas" in sys.argv else []))
