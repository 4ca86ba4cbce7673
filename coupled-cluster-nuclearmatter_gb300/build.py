"""Builds libccx.so (the CUDA engine and its C ABI) for sm_103a, in-tree.

Sources: csrc/*.cu (nvcc) and csrc/*.cpp (host C++), linked into build/libccx.so.
Translation units compile in parallel; only stale objects are rebuilt.  The host
program harness/ccx_run.cpp, which drives the C ABI as the reference's driver drives
its solver, links against it as build/ccx_run.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "build")
INC = os.path.join(os.path.dirname(HERE), "include")
LIB = os.path.join(OUT, "libccx.so")
RUN_SRC = os.path.join(HERE, "harness", "ccx_run.cpp")
RUN = os.path.join(OUT, "ccx_run")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home() -> str:
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found")


def _sources():
    cu = sorted(f for f in os.listdir(SRC) if f.endswith(".cu"))
    cpp = sorted(f for f in os.listdir(SRC) if f.endswith(".cpp"))
    hdr = [os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith((".hpp", ".cuh", ".h"))]
    hdr.append(os.path.join(INC, "ccx.h"))
    return cu, cpp, hdr


def _stale(obj: str, src: str, hdr) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(x) > t for x in [src, *hdr, __file__])


def build(verbose: bool = False) -> str:
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(OUT, exist_ok=True)
    cu, cpp, hdr = _sources()
    common = ["-std=c++17", "-O3", f"-I{SRC}", f"-I{INC}"]
    jobs = []
    objs = []
    for f in cu:
        src, obj = os.path.join(SRC, f), os.path.join(OUT, f + ".o")
        objs.append(obj)
        if _stale(obj, src, hdr):
            jobs.append([nvcc, *ARCH, "-lineinfo", *common, "-Xcompiler", "-fPIC,-ffp-contract=off",
                         "--expt-relaxed-constexpr", "-c", src, "-o", obj])
    for f in cpp:
        src, obj = os.path.join(SRC, f), os.path.join(OUT, f + ".o")
        objs.append(obj)
        if _stale(obj, src, hdr):
            jobs.append(["g++", *common, "-fPIC", "-ffp-contract=off", "-Wall", f"-I{cuda}/include", "-c", src,
                         "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compile failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)

    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        list(ex.map(run, jobs))
    if jobs or not os.path.exists(LIB):
        run([nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"])
    if _stale(RUN, RUN_SRC, [LIB, os.path.join(INC, "ccx.h")]):
        run(["g++", "-std=c++17", "-O2", "-Wall", f"-I{INC}", RUN_SRC, "-o", RUN, f"-L{OUT}", "-lccx",
             "-Wl,-rpath,$ORIGIN"])
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
