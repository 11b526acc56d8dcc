"""Builds the CUDA library (`_build/libdynlight_gb300.so`) for sm_103a with nvcc.

Device code is compiled with --fmad=false and host code with -ffp-contract=off: the bake's f32
arithmetic must round exactly like the reference's (which never fuses a*b+c). The three
translation units compile in parallel; a full build takes about a minute.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libdynlight_gb300.so")
SOURCES = ["dl_bake.cu", "dl_bvh.cu", "dl_host.cpp"]

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "--fmad=false", "--extended-lambda",
          "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math", "-I", os.path.join(HERE, "..", "include")]


def _compile(src):
    obj = os.path.join(OUT, os.path.splitext(src)[0] + ".o")
    cmd = [NVCC] + ARCH + COMMON + ["-c", os.path.join(CSRC, src), "-o", obj]
    if src.endswith(".cpp"):
        cmd += ["-x", "cu"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(verbose=False):
    os.makedirs(OUT, exist_ok=True)
    with ThreadPoolExecutor(len(SOURCES)) as ex:
        results = list(ex.map(_compile, SOURCES))
    for _, err in results:
        if verbose and err.strip():
            print(err, file=sys.stderr)
    objs = [o for o, _ in results]
    cmd = [NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
