"""Build libqkrylov_gb300.so in-tree with nvcc for sm_103a (GB300).

Each translation unit is compiled in parallel, then linked into
qkrylov_gb300/_lib/libqkrylov_gb300.so.  Objects live in qkrylov_gb300/_build/
and are reused when they are newer than every source and header; a stamp
records the host machine so objects from another architecture are rebuilt.

    python -m qkrylov_gb300.build [--force] [--verbose]
"""
import concurrent.futures as cf
import os
import platform
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "libqkrylov_gb300.so")
SOURCES = ["hamiltonian.cu", "spmv_tile.cu", "krylov.cu", "lanczos_dev.cu", "noalloc.cu", "mdot_tc.cu", "block.cu", "basis.cpp", "compile.cpp", "solvers.cpp",
           "c_api.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: set NVCC or put the CUDA toolkit on PATH")


def _flags(src):
    common = ["-std=c++17", "-O3", "-I", os.path.join(ROOT, "include"), "-I", CSRC,
              "-Xcompiler", "-fPIC,-fopenmp,-O2,-Wall,-Wno-unused-function"]
    if src.endswith(".cu"):
        return ARCH + ["-lineinfo", "--extended-lambda", "-Xptxas", "-O3"] + common
    return common


def _headers():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".hpp", ".cuh", ".h"))] + [
        os.path.join(ROOT, "include", "qkrylov_c_api.h")]


def build(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    stamp = os.path.join(BUILD, "machine.txt")
    machine = platform.machine()
    if not os.path.exists(stamp) or open(stamp).read().strip() != machine:
        force = True
    nvcc = _nvcc()
    hdr_time = max(os.path.getmtime(h) for h in _headers())

    def compile_one(src):
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        if not force and os.path.exists(o) and os.path.getmtime(o) > max(os.path.getmtime(s), hdr_time):
            return o, None
        cmd = [nvcc] + _flags(src) + ["-c", s, "-o", o]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            return None, f"{src}:\n{r.stdout}\n{r.stderr}"
        return o, None

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(compile_one, SOURCES))
    errors = [e for _, e in results if e]
    if errors:
        raise RuntimeError("nvcc failed:\n" + "\n".join(errors))
    objs = [o for o, _ in results]
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-Xcompiler", "-fopenmp", "-Xlinker", "-Bsymbolic"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    with open(stamp, "w") as f:
        f.write(machine)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="--verbose" in sys.argv))
