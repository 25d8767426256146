"""The single-header QCS_GPU_CUDA form (qcs_gb300/bundle.py).

* a C89 program that includes the generated header with QCS_IMPLEMENTATION
  compiles under -std=c89 -pedantic and links libqcs_gb300.so;
* without QCS_GPU_CUDA the implementation section refuses to compile;
* without a GPU the program's qc_create fails loudly (no CPU fallback);
  on a GB300 it prepares a Bell pair and finds a Bernstein-Vazirani secret.
"""
import os
import shutil
import subprocess

import pytest

from qcs_gb300 import build as B
from qcs_gb300 import bundle
from qcs_gb300 import capi

PROG = r"""
#define QCS_GPU_CUDA
#define QCS_IMPLEMENTATION
#include "qcs_cuda_single.h"

int main(void) {
  t_q_circuit *c = qc_create(3);
  t_q_circuit *bv;
  if (!c) {
    printf("no device\n");
    return 0;
  }
  qc_h(c, 0);
  qc_cnot(c, 0, 1);
  printf("bell %.6f %.6f %.6f\n", qc_get_probability(c, 0), qc_get_probability(c, 3),
         qc_get_probability(c, 1));
  qc_destroy(c);
  bv = qc_create(6);
  qc_bernstein_vazirani(bv, 19);
  printf("bv %d\n", qc_find_most_likely_state(bv) & 31);
  qc_destroy(bv);
  return 0;
}
"""


def _compile(tmp_path, defines=True):
    if not shutil.which("gcc"):
        pytest.skip("gcc not available")
    lib = B.build()
    bundle.bundle(str(tmp_path / "qcs_cuda_single.h"))
    src = tmp_path / "prog.c"
    src.write_text(PROG if defines else PROG.replace("#define QCS_GPU_CUDA\n", ""))
    exe = tmp_path / "prog"
    libdir = os.path.dirname(lib)
    r = subprocess.run(["gcc", "-std=c89", "-pedantic", "-Wall", "-Wno-long-long",
                        "-I", str(tmp_path), str(src), "-L", libdir, "-lqcs_gb300",
                        f"-Wl,-rpath,{libdir}", "-lm", "-o", str(exe)],
                       capture_output=True, text=True)
    return r, exe


def test_single_header_compiles_links_and_runs(tmp_path):
    r, exe = _compile(tmp_path)
    assert r.returncode == 0, r.stderr
    assert "warning" not in r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0
    if capi.device_count() == 0:
        assert out.stdout.strip() == "no device"
        assert "no usable CUDA device" in out.stderr
    else:
        assert out.stdout.startswith("bell")


def test_single_header_needs_the_mode_define(tmp_path):
    r, _ = _compile(tmp_path, defines=False)
    assert r.returncode != 0
    assert "QCS_GPU_CUDA" in r.stderr


@pytest.mark.gpu
def test_single_header_program_on_the_gpu(tmp_path):
    r, exe = _compile(tmp_path)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    lines = out.stdout.split("\n")
    bell = [float(x) for x in lines[0].split()[1:]]
    assert abs(bell[0] - 0.5) < 1e-6 and abs(bell[1] - 0.5) < 1e-6 and bell[2] < 1e-12
    assert lines[1] == "bv 19"
