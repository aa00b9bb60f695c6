"""Build recipe of the engine's shared library (sm_103a only).

    python refinery-optimizer_gb300/build.py      # or __graft_entry__.build()

Compiles every translation unit under csrc/ in parallel with
``nvcc -gencode arch=compute_103a,code=sm_103a -lineinfo -O3`` and links
``_build/libsih_pdhg.so`` (C ABI of include/sih_pdhg.h, static CUDA runtime).
Rebuilds only what changed since the last build.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(REPO, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(BUILD, "libsih_pdhg.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _headers_mtime() -> float:
    hs = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))
    return max((os.path.getmtime(h) for h in hs), default=0.0)


def _compile(src: str, obj: str) -> None:
    common = ["-O3", "-std=c++17", "-I", INCLUDE, "-I", CSRC]
    if src.endswith(".cu"):
        cmd = [nvcc(), *ARCH, "-lineinfo", *common, "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
               "-c", src, "-o", obj]
    else:
        cmd = ["g++", *common, "-fPIC", "-pthread", "-Wall", "-I", os.path.join(os.path.dirname(nvcc()), "..", "include"),
               "-c", src, "-o", obj]
    subprocess.run(cmd, check=True)


def build(verbose: bool = False) -> str:
    os.makedirs(os.path.join(BUILD, "obj"), exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    hdr = _headers_mtime()
    jobs = []
    objs = []
    for s in srcs:
        o = os.path.join(BUILD, "obj", os.path.basename(s) + ".o")
        objs.append(o)
        if not os.path.exists(o) or os.path.getmtime(o) < max(os.path.getmtime(s), hdr):
            jobs.append((s, o))
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for fut in [ex.submit(_compile, s, o) for s, o in jobs]:
            fut.result()
    if jobs or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        tmp = LIB + ".tmp"
        subprocess.run([nvcc(), *ARCH, "-shared", "-cudart", "static", "-o", tmp, *objs, "-lpthread"], check=True)
        os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
