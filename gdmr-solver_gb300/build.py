"""Builds libgDMR for GB300 (sm_103a) in-tree: gdmr-solver_gb300/lib/libgDMR.so.1.0.1.

Same library name, soname and symlinks as the reference's Makefile
(libgDMR.so.1.0.1, soname libgDMR.so.1, links libgDMR.so.1 and libgDMR.so),
so control programs linked with -lgDMR find it unchanged.  Translation units
compile in parallel with one -gencode; the CUDA runtime is linked statically.

    python gdmr-solver_gb300/build.py [--force] [--jobs N]
"""
from __future__ import annotations

import argparse
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
BUILD = os.path.join(HERE, "_build")
SOURCES = ["gdmr_kernels.cu", "gdmr_tc.cu", "gdmr_engine.cu", "gdmr_api.cu", "gdmr_server.cu", "gdmr_io.cu"]
HEADERS = ["gdmr_kernels.cuh", "gdmr_engine.h"]
PUBLIC = [os.path.join(HERE, "..", "include", h) for h in ("gDMR.h", "gDMRC.h", "gdmr_ext.h")]
MAJOR, MINOR = "1", "0.1"
LIBNAME = f"libgDMR.so.{MAJOR}.{MINOR}"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    return "nvcc"


def lib_path() -> str:
    return os.path.join(LIBDIR, f"libgDMR.so.{MAJOR}")


def _stale(target: str, deps: list) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, jobs: int = 4, verbose: bool = False) -> str:
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(BUILD, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + PUBLIC
    objs = []
    cmds = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            cmds.append([nvcc()] + NVCC_FLAGS + ["-c", s, "-o", o])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return r

    with ThreadPoolExecutor(max_workers=max(1, jobs)) as ex:
        list(ex.map(run, cmds))
    full = os.path.join(LIBDIR, LIBNAME)
    if force or cmds or _stale(full, objs):
        run([nvcc()] + ARCH + ["-shared", "-Xlinker", f"-soname,libgDMR.so.{MAJOR}", "-o", full + ".tmp"] + objs)
        os.replace(full + ".tmp", full)
    for link, target in ((f"libgDMR.so.{MAJOR}", LIBNAME), ("libgDMR.so", f"libgDMR.so.{MAJOR}")):
        p = os.path.join(LIBDIR, link)
        if os.path.islink(p) or os.path.exists(p):
            if os.path.islink(p) and os.readlink(p) == target:
                continue
            os.remove(p)
        os.symlink(target, p)
    return lib_path()


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--jobs", type=int, default=3)
    a = ap.parse_args()
    print(build(force=a.force, jobs=a.jobs, verbose=True))
    sys.exit(0)
