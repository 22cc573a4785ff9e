"""Build recipe for libfastlem_gb300.so (the C-ABI library).

CUDA sources are compiled for sm_103a only; host C++ with g++.  Both keep every
floating-point operation as written (`-fmad=false`, `-ffp-contract=off`), because the
solve must reproduce fastlem's rounding bit for bit.  Objects are compiled in
parallel and linked with the CUDA runtime statically, so the library only needs the
driver at run time.  Output: fastlem_gb300/_build/<machine>/libfastlem_gb300.so (git-ignored,
built in-tree on every machine that runs it).
"""
import os
import platform
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT_DIR = os.path.join(PKG, "_build", platform.machine())
LIB = os.path.join(OUT_DIR, "libfastlem_gb300.so")
INCLUDE = os.path.join(ROOT, "include")

CUDA_SOURCES = ["solver.cu", "receivers.cu", "basin.cu", "noalloc.cu", "lake_rank.cu",
                "ordering.cu", "interp_gpu.cu"]
CXX_SOURCES = ["builder.cpp", "prim_rank.cpp", "server.cpp", "interp.cpp"]
HEADERS = ["rng.h", "common.cuh", "kernels.h", "fold.cuh", "delaunay.h", "ordering.h",
           "interp.h", "expansion.cuh", "interp_query.cuh"]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xptxas", "-v",
                     "-Xcompiler", "-fPIC,-ffp-contract=off", "-I", INCLUDE, "-I", CSRC]
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-pthread",
             "-I", INCLUDE, "-I", CSRC]


def _nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build fastlem_gb300")


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd, log):
    r = subprocess.run(cmd, capture_output=True, text=True)
    with open(log, "w") as f:
        f.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
    if r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError("build step failed: " + " ".join(cmd))


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    nvcc = _nvcc()
    headers = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "fastlem_gb300.h")]
    jobs, objs = [], []
    for src in CUDA_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT_DIR, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append(([nvcc, *NVCC_FLAGS, "-c", s, "-o", o], o + ".log"))
    cuda_inc = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "include")
    for src in CXX_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT_DIR, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append((["g++", *CXX_FLAGS, "-I", cuda_inc, "-c", s, "-o", o], o + ".log"))
    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        list(ex.map(lambda j: _run(*j), jobs))
    if force or jobs or _stale(LIB, objs):
        tmp = LIB + ".tmp%d" % os.getpid()
        _run([nvcc, *ARCH, "-shared", "-cudart", "static", "-o", tmp, *objs, "-lpthread"],
             os.path.join(OUT_DIR, "link.log"))
        os.replace(tmp, LIB)
    if verbose:
        for src in CUDA_SOURCES:
            with open(os.path.join(OUT_DIR, src + ".o.log")) as f:
                print(f.read())
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
