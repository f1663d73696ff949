"""Build libsgmres.so in-tree (``schwarz_gmres_dashboard_gb300/_build/``) with nvcc
for sm_103a.  Translation units compile in parallel; an object is rebuilt only
when its source or any header is newer.  No CMake, no torch extension machinery.

    python -m schwarz_gmres_dashboard_gb300.build      # or build() from Python
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libsgmres.so")
CLI = os.path.join(BUILD, "schwarz_solve")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code without contracted multiply-adds: the generators and the host
# set-up give the same bits on x86-64 and aarch64 (where FMA is always there)
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler",
          "-ffp-contract=off", "-I", INCLUDE, "-I", CSRC]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libsgmres")


def _headers():
    return glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))


def _stale(obj: str, src: str, hdr_mtime: float) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return t < os.path.getmtime(src) or t < hdr_mtime


def build(verbose: bool = False, jobs: int | None = None) -> str:
    """Compile every CUDA/C++ source of the package for sm_103a and link
    libsgmres.so.  Returns the library path."""
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    hdr_mtime = max([os.path.getmtime(h) for h in _headers()] + [0.0])
    # objects compiled with other flags are stale too
    stamp = os.path.join(BUILD, "flags.txt")
    flags = " ".join(ARCH + COMMON)
    if not os.path.exists(stamp) or open(stamp).read() != flags:
        for o in glob.glob(os.path.join(BUILD, "*.o")):
            os.remove(o)
        with open(stamp, "w") as f:
            f.write(flags)
    objs, todo = [], []
    for s in srcs:
        o = os.path.join(BUILD, os.path.basename(s) + ".o")
        objs.append(o)
        if _stale(o, s, hdr_mtime):
            todo.append((s, o))

    def compile_one(item):
        s, o = item
        cmd = [nvcc, *ARCH, *COMMON, "-c", s, "-o", o]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {os.path.basename(s)}:\n{r.stdout}\n{r.stderr}")
        return r.stderr

    if todo:
        with cf.ThreadPoolExecutor(max_workers=jobs or min(len(todo), os.cpu_count() or 4)) as ex:
            for msg in ex.map(compile_one, todo):
                if verbose and msg:
                    print(msg, file=sys.stderr)
    if todo or not os.path.exists(LIB):
        cmd = [nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-ldl"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    # the schwarz_solve CLI, linked against the library next to it
    cli_src = os.path.join(CSRC, "cli", "schwarz_solve.cpp")
    if (not os.path.exists(CLI) or os.path.getmtime(CLI) < os.path.getmtime(cli_src)
            or os.path.getmtime(CLI) < os.path.getmtime(LIB)):
        cxx = shutil.which("g++") or "g++"
        cmd = [cxx, "-O2", "-std=c++17", "-I", INCLUDE, cli_src, "-o", CLI, "-L", BUILD,
               "-lsgmres", "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"CLI build failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
