"""In-tree build of libdoonengine.so (CUDA kernels for sm_103a + the DN_* host C layer).

Used by ``__graft_entry__.build()`` and by ``doonengine_gb300.load()``.  Host C is compiled with
``-ffp-contract=off`` and the CUDA unit with ``--fmad=false`` and IEEE division / square root, so
that every floating-point operation is rounded on its own, as the bit-exact ray traversal needs.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(OUT, "libdoonengine.so")
INCLUDE = os.path.join(ROOT, "include")

NVCC = os.environ.get("NVCC", "nvcc")
CC = os.environ.get("CC", "gcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_FLAGS = ARCH + ["-lineinfo", "-O3", "--fmad=false", "-prec-div=true", "-prec-sqrt=true",
                     "-ftz=false", "-std=c++17", "-Xcompiler", "-fPIC", "-I" + INCLUDE, "-I" + CSRC]
# extra nvcc defines for tuning experiments, e.g. DN_NVCC_EXTRA="-DDN_STREAM_MIN_BLOCKS=5"
CUDA_FLAGS += [f for f in os.environ.get("DN_NVCC_EXTRA", "").split() if f.startswith("-D")]
C_FLAGS = ["-O2", "-fPIC", "-fno-semantic-interposition", "-std=gnu11", "-ffp-contract=off", "-fno-fast-math", "-Wall",
           "-Wno-unused-function", "-I" + INCLUDE]

CU_SOURCES = ["dn_cuda.cu", "dn_batch.cu", "dn_shapes.cu"]
C_SOURCES = ["voxel.c", "dn_math.c", "dn_scenes.c", "voxvol.c", "dn_serve.c", "voxelShapes.c", "dn_residency.c"]
HEADERS = sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))) + [
    os.path.join(INCLUDE, "dn_cuda.h"), os.path.join(INCLUDE, "DoonEngine", "voxel.h"),
    os.path.join(INCLUDE, "DoonEngine", "globals.h"), os.path.join(INCLUDE, "DoonEngine", "dn_math.h"),
    os.path.join(INCLUDE, "DoonEngine", "serve.h"), os.path.join(INCLUDE, "DoonEngine", "voxelShapes.h")]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def build(force=False, verbose=False):
    """Compile every translation unit (in parallel) and link libdoonengine.so; returns its path."""
    os.makedirs(OUT, exist_ok=True)
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + HEADERS):
            jobs.append([NVCC] + CUDA_FLAGS + ["-c", s, "-o", o])
    for src in C_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + HEADERS):
            jobs.append([CC] + C_FLAGS + ["-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out:
                sys.stdout.write(out)
    if force or jobs or _stale(LIB, objs):
        _run([NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lm", "-lpthread"])
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
