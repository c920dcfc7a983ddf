"""Builds libgbrt.so in-tree with nvcc for sm_103a only.

Each .cu file compiles in parallel to an object; the objects link into one
shared library with the CUDA runtime linked statically.  Files listed in
EXACT_FP compile with --fmad=false: their float arithmetic must round like
the reference's scalar CPU code (no fused multiply-add).
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgbrt.so")

SOURCES = ["capi.cu", "bvh_build.cu", "traverse.cu", "pathtrace.cu", "guiding.cu", "mesh.cu", "texture_eval.cu"]
EXACT_FP = {"traverse.cu", "pathtrace.cu", "texture_eval.cu"}
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    p = shutil.which("nvcc")
    if p:
        return p
    for c in ("/usr/local/cuda/bin/nvcc",):
        if os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libgbrt.so")


def _compile(src):
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
           "-I", os.path.join(ROOT, "include"), "-I", CSRC, "-c", os.path.join(CSRC, src), "-o", obj]
    if src in EXACT_FP:
        cmd.insert(1, "--fmad=false")
    if os.environ.get("GBRT_PTXAS_VERBOSE"):
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(_compile, SOURCES))
    if verbose:
        for _, err in results:
            if err:
                print(err, file=sys.stderr)
    objs = [o for o, _ in results]
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-cudart", "static"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
