"""The allocation-free device dot product.

qkrylov_vector_dot_device_f64_noalloc serves callers that cannot let a
library call cudaMalloc (applications that own the GPU's memory in their own
pool or under a hard cap, latency-critical loops that cannot take cudaMalloc's
implicit synchronisation).  It must give the result of the allocating
qkrylov_vector_dot_device_f64 on the same device vectors, call after call,
since every call reuses one fixed scratch array, and it must refuse sizes
beyond that array's limit of 8192 * 16384 complex elements.

This file is named to be collected last, so a run stopping at the first
failure has run every other test before it.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL64 = 1e-13  # the FP64 tolerance of the SpMV/BLAS parity tests
MAX_ELEMENTS = 8192 * 16384


def _cudart():
    from test_gpu_spmv import _cudart as c
    return c()


def _to_device(cudart, a):
    p = ctypes.c_void_p()
    assert cudart.cudaMalloc(ctypes.byref(p), max(16, a.nbytes)) == 0
    assert cudart.cudaMemcpy(p, a.ctypes.data_as(ctypes.c_void_p), a.nbytes, 1) == 0
    return p


def _dot(fn, dx, dy, n):
    out = np.zeros(2)
    rc = fn(dx, dy, n, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), None)
    return rc, complex(out[0], out[1])


def test_noalloc_dot_matches_allocating_dot_on_consecutive_calls(qk):
    L = qk.lib()
    cudart = _cudart()
    rng = np.random.default_rng(2024)
    # two calls in a row on different data (the second one reuses the scratch the first one filled)
    for n in (3_000_001, 40_000):
        x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
        y = rng.standard_normal(n) + 1j * rng.standard_normal(n)
        dx, dy = _to_device(cudart, x), _to_device(cudart, y)
        try:
            rc_new, v_new = _dot(L.qkrylov_vector_dot_device_f64_noalloc, dx, dy, n)
            rc_old, v_old = _dot(L.qkrylov_vector_dot_device_f64, dx, dy, n)
        finally:
            cudart.cudaFree(dx)
            cudart.cudaFree(dy)
        assert rc_new == 0 and rc_old == 0
        scale = np.linalg.norm(x) * np.linalg.norm(y)
        assert abs(v_new - v_old) <= RTOL64 * scale
        assert abs(v_new - np.vdot(x, y)) <= RTOL64 * scale


def test_noalloc_dot_fills_every_scratch_slot_on_a_stream(qk):
    """n = 8192 * 16384: all 16384 partial slots are written, the last one next
    to the result slot; on a stream the caller created."""
    L = qk.lib()
    cudart = _cudart()
    n = MAX_ELEMENTS
    i = np.arange(n, dtype=np.int64)
    y = ((i % 7) - 3).astype(np.float64) + 1j * ((i % 5) - 2).astype(np.float64)
    x = np.ones(n, dtype=np.complex128)
    exact = complex(float(((i % 7) - 3).sum()), float(((i % 5) - 2).sum()))  # sum of conj(1) * y
    del i
    dx, dy = _to_device(cudart, x), _to_device(cudart, y)
    del x, y
    st = ctypes.c_void_p()
    assert cudart.cudaStreamCreate(ctypes.byref(st)) == 0
    try:
        out = np.zeros(2)
        for _ in range(2):
            assert L.qkrylov_vector_dot_device_f64_noalloc(dx, dy, n, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                                           st) == 0
            assert complex(out[0], out[1]) == exact  # small integers: every partial sum is exact
    finally:
        cudart.cudaStreamDestroy(st)
        cudart.cudaFree(dx)
        cudart.cudaFree(dy)


def test_noalloc_dot_rejects_sizes_beyond_its_scratch(qk):
    L = qk.lib()
    out = np.zeros(2)
    dp = out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    # rejected before any device access: the pointers are never dereferenced
    rc = L.qkrylov_vector_dot_device_f64_noalloc(ctypes.c_void_p(16), ctypes.c_void_p(16), MAX_ELEMENTS + 1, dp, None)
    assert rc == qk.ERROR_INVALID_ARG
    assert b"exceeds" in L.qkrylov_last_error()
    # n = 0 is the warm-up call: it looks up the scratch array and loads the kernels, and computes nothing
    assert L.qkrylov_vector_dot_device_f64_noalloc(None, None, 0, dp, None) == 0 and out[0] == 0.0
