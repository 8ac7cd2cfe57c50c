"""Device-vector reductions of the C ABI against numpy (FP64) and against the
FP64 sum of FP32 data (compensated FP32 kernel)."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL64 = 1e-13


def _dev(cudart, a):
    p = ctypes.c_void_p()
    assert cudart.cudaMalloc(ctypes.byref(p), max(16, a.nbytes)) == 0
    assert cudart.cudaMemcpy(p, a.ctypes.data_as(ctypes.c_void_p), a.nbytes, 1) == 0
    return p


@pytest.mark.parametrize("n", [1, 1000, 1 << 20, 3_000_001])
def test_dot_device(qk, n):
    from test_gpu_spmv import _cudart
    cudart = _cudart()
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    y = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    dx, dy = _dev(cudart, x), _dev(cudart, y)
    x32, y32 = x.astype(np.complex64), y.astype(np.complex64)
    fx, fy = _dev(cudart, x32), _dev(cudart, y32)
    try:
        out = np.zeros(2)
        dp = out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        assert qk.lib().qkrylov_vector_dot_device_f64(dx, dy, n, dp, None) == 0
        ref = np.vdot(x, y)
        assert abs(complex(*out) - ref) <= RTOL64 * np.sqrt(n) * np.linalg.norm(x) * np.linalg.norm(y) / np.sqrt(n)
        assert qk.lib().qkrylov_vector_dot_device_f32(fx, fy, n, dp, None) == 0
        ref32 = np.vdot(x32.astype(np.complex128), y32.astype(np.complex128))  # exact products of the FP32 data
        assert abs(complex(*out) - ref32) <= 1e-12 * np.linalg.norm(x) * np.linalg.norm(y)
    finally:
        for p in (dx, dy, fx, fy):
            cudart.cudaFree(p)
    assert qk.lib().qkrylov_vector_dot_device_f64(None, None, 0, dp, None) == 0 and out[0] == 0.0
    assert qk.lib().qkrylov_vector_dot_device_f64(None, None, 5, dp, None) == qk.ERROR_INVALID_ARG
