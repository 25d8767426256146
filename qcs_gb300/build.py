"""Build libqcs_gb300.so in-tree (nvcc for sm_103a, gcc for the C89 API).

    python -m qcs_gb300.build            # library only
    python -m qcs_gb300.build --verbose  # also print ptxas register/smem use

Objects go to qcs_gb300/_build/ and the library to qcs_gb300/libqcs_gb300.so
(both git-ignored).  Translation units compile in parallel; a full build
takes well under a minute.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libqcs_gb300.so")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["state.cu", "gates.cu", "readout.cu", "blocks.cu", "blocks_tc.cu",
              "batch.cu", "mlp.cu", "noalloc.cu"]
CPP_SOURCES = ["fusion.cpp", "costmodel.cpp"]
C_SOURCES = ["qcs_api.c"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd, verbose):
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + p.stdout + p.stderr)
    if verbose and (p.stdout or p.stderr):
        sys.stderr.write(p.stdout + p.stderr)


def _stale(obj, srcs):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(s) > t for s in srcs)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    # objects built on another machine type (x86 here, aarch64 on the GPU
    # host) are never reused
    import platform
    stamp = os.path.join(BUILD, "ARCH")
    arch = platform.machine()
    if not os.path.exists(stamp) or open(stamp).read().strip() != arch:
        force = True
        with open(stamp, "w") as f:
            f.write(arch + "\n")
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    jobs = []
    for f in CU_SOURCES:
        src = os.path.join(CSRC, f)
        if not os.path.exists(src):
            continue
        obj = os.path.join(BUILD, f + ".o")
        cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-c", src, "-o", obj,
               "-I", INCLUDE, "-I", CSRC, "-Xcompiler", "-fPIC,-ffp-contract=off",
               "--expt-relaxed-constexpr"]
        if verbose:
            cmd += ["-Xptxas", "-v"]
        jobs.append((obj, [src] + headers, cmd))
    for f in CPP_SOURCES:
        src = os.path.join(CSRC, f)
        if not os.path.exists(src):
            continue
        obj = os.path.join(BUILD, f + ".o")
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-c", src, "-o", obj,
               "-I", INCLUDE, "-I", CSRC]
        jobs.append((obj, [src] + headers, cmd))
    for f in C_SOURCES:
        src = os.path.join(HOST, f)
        obj = os.path.join(BUILD, f + ".o")
        cmd = ["gcc", "-std=c89", "-pedantic", "-Wall", "-Wextra", "-Wno-long-long", "-O2",
               "-fPIC", "-ffp-contract=off", "-c", src, "-o", obj, "-I", INCLUDE]
        jobs.append((obj, [src] + headers, cmd))
    todo = [j for j in jobs if force or _stale(j[0], j[1])]
    with cf.ThreadPoolExecutor(max_workers=min(8, max(1, len(todo)))) as ex:
        list(ex.map(lambda j: _run(j[2], verbose), todo))
    objs = [j[0] for j in jobs]
    if force or todo or not os.path.exists(LIB) or _stale(LIB, objs):
        tmp = LIB + ".tmp"
        _run([nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart_static", "-lpthread", "-ldl",
              "-lrt", "-lm"], verbose)
        os.replace(tmp, LIB)
    return LIB


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--verbose", action="store_true")
    ap.add_argument("--force", action="store_true")
    a = ap.parse_args()
    print(build(verbose=a.verbose, force=a.force))


if __name__ == "__main__":
    main()
