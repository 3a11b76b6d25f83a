"""Build libsvdb_gb300.so in-tree: C host layer (gcc) + CUDA layer (nvcc,
sm_103a only), objects compiled in parallel, one shared library linked
with the static CUDA runtime.

    python simple-vector-db_gb300/build.py [-v] [--force]
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
LIB = os.path.join(OUT, "libsvdb_gb300.so")
PERCALL_LIB = os.path.join(OUT, "libsvdb_percall.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"

C_SOURCES = ["svdb_store.c", "svdb_kdtree.c", "svdb_api.c", "svdb_server.c", "svdb_combine.c"]
CU_SOURCES = ["dev_store.cu", "dev_search.cu", "dev_kd.cu", "dev_gemm.cu", "dev_noalloc.cu", "dev_ragged.cu", "dev_uuid.cu", "dev_kdm.cu", "dev_decode.cu", "dev_loop.cu"]


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    inc = os.path.join(ROOT, "include")
    hs += [os.path.join(inc, f) for f in os.listdir(inc) if f.endswith(".h")]
    return hs


def _stale(obj: str, src: str, deps: list[str]) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(p) > t for p in [src, *deps, __file__])


def _run(cmd: list[str], verbose: bool) -> None:
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose and (r.stdout or r.stderr):
        print(r.stdout + r.stderr, flush=True)


def build(verbose: bool = False, force: bool = False, ptxas_verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    deps = _headers()
    inc = ["-I" + CSRC, "-I" + os.path.join(ROOT, "include")]
    jobs = []
    objs = []
    for f in C_SOURCES:
        src, obj = os.path.join(CSRC, f), os.path.join(OUT, f + ".o")
        objs.append(obj)
        if force or _stale(obj, src, deps):
            jobs.append(["gcc", "-std=c11", "-O2", "-fPIC", "-fvisibility=hidden", "-Wall", "-Wextra",
                         "-Wno-unused-parameter", "-D_GNU_SOURCE", *inc, "-c", src, "-o", obj])
    for f in CU_SOURCES:
        src, obj = os.path.join(CSRC, f), os.path.join(OUT, f + ".o")
        objs.append(obj)
        if force or _stale(obj, src, deps):
            cmd = [nvcc, ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-fvisibility=hidden",
                   "--expt-relaxed-constexpr", *inc, "-c", src, "-o", obj]
            if ptxas_verbose:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(lambda c: _run(c, verbose or ptxas_verbose), jobs))
    if jobs or not os.path.exists(LIB):
        _run([nvcc, ARCH, "-shared", "-o", LIB, *objs, "-Xlinker", "-Bsymbolic", "-lpthread", "-ldl", "-lrt"],
             verbose)
    # the per-call timing harness (bench.py --workload percall): its own small library
    drv_src = os.path.join(CSRC, "percall_driver.c")
    if force or _stale(PERCALL_LIB, drv_src, deps):
        _run(["gcc", "-std=c11", "-O2", "-fPIC", "-shared", "-fvisibility=hidden", "-Wall", "-Wextra", "-D_GNU_SOURCE",
              *inc, "-o", PERCALL_LIB, drv_src, "-lpthread"], verbose)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="--force" in sys.argv, ptxas_verbose="--ptxas" in sys.argv))
