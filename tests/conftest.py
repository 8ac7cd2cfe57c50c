import glob
import os
import subprocess
import sys

import numpy as np
import pytest

# The oracle's reductions are deterministic per thread count; one thread
# reproduces the order the golden fixtures were generated with.
os.environ["OMP_NUM_THREADS"] = "1"

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TESTS = os.path.join(ROOT, "tests")
GOLDEN = os.path.join(TESTS, "golden")
for p in (ROOT, TESTS):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the library's kernels)")


def golden_names():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz"))
                  if not os.path.basename(p).startswith("capi_"))


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False))


def golden_terms(g):
    """Rebuild the OpSum term list stored in a fixture."""
    terms, k = [], 0
    for c, nf in zip(g["coeff"], g["nfac"]):
        facs = [(str(g["ops"][k + j]), int(g["sites"][k + j])) for j in range(int(nf))]
        k += int(nf)
        terms.append((complex(c), facs))
    return terms


@pytest.fixture(scope="session")
def oracle():
    """The oracle restatement (oracle/_build/libqko.so), built on demand."""
    from oracle_ctypes import Oracle, available
    if not available("qko"):
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "oracle"], check=True)
    return Oracle("qko")


@pytest.fixture(scope="session")
def qk():
    """The GPU library's Python mirror, built on demand (nvcc cross-compiles
    without a GPU)."""
    from qkrylov_gb300 import build as b
    if not os.path.exists(b.LIB):
        b.build()
    import qkrylov_gb300
    qkrylov_gb300.lib()
    return qkrylov_gb300


from models import make_model  # noqa: E402,F401  (re-exported for the tests)

