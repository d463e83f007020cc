"""Compile libgbpt.so (CUDA kernels for sm_103a + C ABI) in-tree.

Translation units are compiled in parallel with nvcc and linked into
``cudapt_gb300/_build/libgbpt.so``.  Kernels are built with -fmad=false so
that no multiply-add is contracted behind the float contract the CPU oracle
follows; host code uses -ffp-contract=off for the same reason (GCC on Arm
contracts by default).
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libgbpt.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["kernels_wave.cu", "kernels_adapt.cu", "api.cu", "noalloc.cu", "image.cu", "texture.cu", "mlp.cu",
           "bvh_build.cpp", "server.cpp"]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.sep not in c or os.path.exists(c)):
            return c
    return "nvcc"


def _cmd(src, obj):
    host = "-fPIC,-ffp-contract=off,-O2,-fno-fast-math"
    base = [_nvcc(), "-c", os.path.join(CSRC, src), "-o", obj, "-std=c++17", "-O3", "-Xcompiler", host]
    if src.endswith(".cu"):
        return base + ARCH + ["-lineinfo", "-fmad=false", "-Xptxas", "-O3", "--extended-lambda"]
    return base + ["-x", "c++"]


def _stale(obj, src):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(HERE, "..", "include", "gbpt.h")]
    return any(os.path.exists(d) and os.path.getmtime(d) > t for d in deps + [os.path.join(CSRC, src)])


def build(force=False, verbose=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    objs, jobs = [], []
    for src in SOURCES:
        obj = os.path.join(OUT_DIR, src.rsplit(".", 1)[0] + ".o")
        objs.append(obj)
        if force or _stale(obj, src):
            jobs.append(_cmd(src, obj))

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compile failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        return r.stderr

    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        for err in ex.map(run, jobs):
            if verbose and err:
                print(err)
    if jobs or not os.path.exists(LIB):
        link = [_nvcc(), "-shared", "-o", LIB] + objs + ARCH + ["-lcudart", "-lpthread"]
        r = subprocess.run(link, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + " ".join(link) + "\n" + r.stdout + r.stderr)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
