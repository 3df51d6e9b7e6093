"""Builds libam.so (the CUDA kernels + C ABI) in-tree for sm_103a.

    python -m adaptivemerging_gb300.build

Translation units are compiled in parallel; --fmad=false keeps every FP64
expression un-contracted (bit-identical to the reference arithmetic) and
-ffp-contract=off does the same for the host code on aarch64 hosts.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "libam.so")
BUILD = os.path.join(HERE, "_build")
SOURCES = ["collide.cu", "solve.cu", "step.cu", "capi.cu", "pgs_fast.cu", "merging.cu", "gs_exact.cu", "batch.cu", "learned.cu", "state.cu"]
# translation units that may contract a*b+c (the coloured FP64 solve and the
# FP32 batched and learned paths; none of them is part of the bit-exact path)
FMA_OK = {"pgs_fast.cu", "batch.cu", "learned.cu"}
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-std=c++17", "-O3", "-lineinfo", "--fmad=false", "-Xcompiler", "-fPIC,-ffp-contract=off",
         "-diag-suppress", "550"]


def nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.exists(c) or c == "nvcc"):
            return c
    return "nvcc"


def _stale(obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False):
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".hpp", ".cuh"))]
    headers.append(os.path.join(HERE, "..", "include", "am.h"))
    jobs = []
    objs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + headers):
            fl = [f if not (src in FMA_OK and f == "--fmad=false") else "--fmad=true" for f in FLAGS]
            jobs.append([nvcc()] + fl + ARCH + ["-c", s, "-o", o])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        return r.stderr

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        for msg in ex.map(run, jobs):
            if verbose and msg.strip():
                print(msg, file=sys.stderr)
    if force or jobs or not os.path.exists(OUT) or _stale(OUT, objs):
        link = [nvcc(), "-shared"] + ARCH + objs + ["-o", OUT, "-lcudart"]
        r = subprocess.run(link, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    return OUT


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
