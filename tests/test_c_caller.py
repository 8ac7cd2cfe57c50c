"""The C ABI as compiled code sees it: the reference's own C API test
(tests/test_c_api.cpp of the reference) compiled unchanged against this
library's include/ and linked to libqkrylov_gb300.so (prototype and link
compatibility; CPU, where the reference tree is present), and a C11 program
of this repository walking the same flow on the GPU (tests/c_caller/flow.c)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import load_golden

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(ROOT, "include")
LIBDIR = os.path.join(ROOT, "qkrylov_gb300", "_lib")
REFERENCE = os.environ.get("QKRYLOV_REFERENCE", "/root/reference")


def _lib():
    if not os.path.exists(os.path.join(LIBDIR, "libqkrylov_gb300.so")):
        pytest.skip("libqkrylov_gb300.so not built")


def _build(compiler, src, out, extra):
    cmd = [compiler] + extra + ["-I", INC, src, "-o", out, "-L", LIBDIR, "-lqkrylov_gb300", "-lm",
                                "-Wl,-rpath," + LIBDIR]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr


def test_reference_c_api_test_compiles_and_links(tmp_path):
    src = os.path.join(REFERENCE, "tests", "test_c_api.cpp")
    if not os.path.exists(src):
        pytest.skip("reference source tree not present")
    _lib()
    if not shutil.which("g++"):
        pytest.skip("g++ not found")
    _build("g++", src, str(tmp_path / "ref_c_api_test"), ["-std=c++17", "-O1"])


def test_c_flow_program_compiles_as_c11(tmp_path):
    _lib()
    if not shutil.which("gcc"):
        pytest.skip("gcc not found")
    _build("gcc", os.path.join(ROOT, "tests", "c_caller", "flow.c"), str(tmp_path / "flow"),
           ["-std=c11", "-O1", "-Wall", "-Werror"])


@pytest.mark.gpu
def test_c_flow_program_runs(tmp_path):
    _lib()
    exe = str(tmp_path / "flow")
    _build("gcc", os.path.join(ROOT, "tests", "c_caller", "flow.c"), exe, ["-std=c11", "-O1"])
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    vals = dict(line.split() for line in r.stdout.splitlines() if line.strip())
    g = load_golden("heis_L10_pbc_sz0")
    e_ref = float(g["lanczos_E0"])
    assert abs(float(vals["E0_f64"]) - e_ref) <= 1e-10 * abs(e_ref)
    assert abs(float(vals["E0_float"]) - e_ref) <= 1e-5 * abs(e_ref)
    assert abs(float(vals["E1_davidson"]) - float(g["davidson_evals"][1])) <= 1e-4
