"""Single-header form of the QCS API in QCS_GPU_CUDA mode.

QCS ships as one generated header (scripts/bundle.py:125-240): the public
declarations, then every implementation file under `#ifdef
QCS_IMPLEMENTATION`, with the parallel mode picked by a define before the
include (QCS_MULTI_THREAD, QCS_CPU_OPENMP, QCS_GPU_OPENCL, QCS_SIMD_ONLY).
This script writes the QCS_GPU_CUDA part of such a header: the declarations
of include/qcs.h, include/qcs_cuda.h and include/qcs_ext.h, and the C89 host
layer (host/qcs_api.c) as the implementation.  The compute stays in the
prebuilt libqcs_gb300.so, which the program links:

    #define QCS_GPU_CUDA
    #define QCS_IMPLEMENTATION
    #include "qcs_cuda_single.h"

    gcc -std=c89 prog.c -L<dir> -lqcs_gb300 -Wl,-rpath,<dir> -lm

The implementation section refuses to compile without QCS_GPU_CUDA, so a
program cannot end up on this header's host layer by accident.  In a merged
header that carries the CPU modes too, this section sits in the
`#ifdef QCS_GPU_CUDA` branch and the reference's own src/*.c in the `#else`
branch: both define the qc_* functions.

Usage: python -m qcs_gb300.bundle [output path]  (default:
qcs_gb300/_build/qcs_cuda_single.h)
"""
from __future__ import annotations

import os
import re
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
HEADERS = ("include/qcs.h", "include/qcs_cuda.h", "include/qcs_ext.h")
IMPLEMENTATION = ("qcs_gb300/host/qcs_api.c",)
DEFAULT_OUT = os.path.join(PKG, "_build", "qcs_cuda_single.h")

# project headers are pasted in place, so their #include lines go
_LOCAL_INCLUDE = re.compile(r'^\s*#\s*include\s+"[^"]*(qcs|qcs_cuda|qcs_ext)\.h"\s*$')


def _strip_local_includes(text: str) -> str:
    return "\n".join(l for l in text.splitlines() if not _LOCAL_INCLUDE.match(l)) + "\n"


def bundle_text() -> str:
    parts = ["""/*
 * qcs_cuda_single.h -- QCS single-header library, QCS_GPU_CUDA mode.
 * Generated by qcs_gb300/bundle.py; do not edit.
 *
 * Declarations: the unchanged QCS API (qcs.h), the C ABI of the GB300
 * backend (qcs_cuda.h) and its additive extensions (qcs_ext.h).
 * Implementation (one C file defines QCS_IMPLEMENTATION, with QCS_GPU_CUDA):
 * the C89 host layer; link libqcs_gb300.so for the device side.
 */
#ifndef QCS_CUDA_SINGLE_H
#define QCS_CUDA_SINGLE_H
"""]
    for h in HEADERS:
        with open(os.path.join(ROOT, h)) as f:
            parts.append(f"\n/* ---- {h} ---- */\n")
            parts.append(_strip_local_includes(f.read()))
    parts.append("""
#ifdef QCS_IMPLEMENTATION
#ifndef QCS_GPU_CUDA
#error "qcs_cuda_single.h implements the QCS_GPU_CUDA mode only: define QCS_GPU_CUDA"
#endif
""")
    for c in IMPLEMENTATION:
        with open(os.path.join(ROOT, c)) as f:
            parts.append(f"\n/* ---- {c} ---- */\n")
            parts.append(_strip_local_includes(f.read()))
    parts.append("\n#endif /* QCS_IMPLEMENTATION */\n#endif /* QCS_CUDA_SINGLE_H */\n")
    return "".join(parts)


def bundle(out: str = DEFAULT_OUT) -> str:
    os.makedirs(os.path.dirname(os.path.abspath(out)), exist_ok=True)
    text = bundle_text()
    tmp = out + ".tmp"
    with open(tmp, "w") as f:
        f.write(text)
    os.replace(tmp, out)
    return out


if __name__ == "__main__":
    print(bundle(sys.argv[1] if len(sys.argv) > 1 else DEFAULT_OUT))
