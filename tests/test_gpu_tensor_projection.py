"""Tall-skinny projections <V_j, W_o> of FP32 complex device vectors: the
compensated CUDA-core kernel (FP64-accurate sums) and the tcgen05 tensor-core
kernel (3xTF32 products, FP32 sums of about a thousand products added in
FP64), against FP64 sums of the same FP32 data.  These are the Davidson
solver's projected-matrix and Gram-Schmidt products
(src/solvers/davidson.cpp:143-150, 213-223)."""
import ctypes

import numpy as np
import pytest

import models as M
from conftest import make_model

pytestmark = pytest.mark.gpu

CUDA_RTOL = 1e-12  # compensated FP32 sums: FP64-level, relative to sum |v||w|
TC_RTOL = 2e-6     # 3xTF32 products, FP32 partial sums of about a thousand products
FAST_RTOL = 1e-6   # FP32 sums over runs of 32 products, folded into float-float sums


def _cudart():
    from test_gpu_spmv import _cudart as c
    return c()


def _dev(cudart, a):
    p = ctypes.c_void_p()
    assert cudart.cudaMalloc(ctypes.byref(p), max(16, a.nbytes)) == 0
    assert cudart.cudaMemcpy(p, a.ctypes.data_as(ctypes.c_void_p), a.nbytes, 1) == 0
    return p


def _mdot(qk, dv, dw, n, method):
    k, nw = len(dv), len(dw)
    out = np.zeros(2 * k * nw)
    va = (ctypes.c_void_p * k)(*[p.value for p in dv])
    wa = (ctypes.c_void_p * nw)(*[p.value for p in dw])
    rc = qk.lib().qkrylov_vector_mdot_device_f32(va, k, wa, nw, n, method,
                                                  out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), None)
    return rc, out.view(np.complex128).reshape(nw, k)


# (the ring depth of the tensor-core kernel runs from 14 stages at k <= 16 to 1 at k > 96)
@pytest.mark.parametrize("n,k,nw", [(1_000_003, 36, 4), (4097, 1, 1), (5, 3, 2), (70_000, 128, 3), (300_000, 17, 4),
                                    (2_000_001, 64, 4), (123_457, 100, 2), (33, 8, 1)])
def test_projection_kernels_against_fp64(qk, n, k, nw):
    cudart = _cudart()
    rng = np.random.default_rng(n + k)
    V = (rng.standard_normal((k, n)) + 1j * rng.standard_normal((k, n))).astype(np.complex64)
    Wv = (rng.standard_normal((nw, n)) + 1j * rng.standard_normal((nw, n))).astype(np.complex64)
    dv = [_dev(cudart, V[j]) for j in range(k)]
    dw = [_dev(cudart, Wv[o]) for o in range(nw)]
    try:
        ref = np.conj(V.astype(np.complex128)) @ Wv.astype(np.complex128).T  # [k, nw]
        scale = np.abs(V).astype(np.float64) @ np.abs(Wv).astype(np.float64).T
        for method, tol in ((0, CUDA_RTOL), (1, TC_RTOL), (2, FAST_RTOL)):
            first = None
            for _ in range(2):  # a second call on the same data gives the same numbers
                rc, got = _mdot(qk, dv, dw, n, method)
                assert rc == 0, qk.lib().qkrylov_last_error()
                err = np.abs(got.T - ref) / scale
                assert err.max() <= tol, (method, err.max())
                if first is None:
                    first = got
                else:
                    assert np.array_equal(got, first)
    finally:
        for p in dv + dw:
            cudart.cudaFree(p)


@pytest.mark.parametrize("n,k,nw,acc", [(1_000_003, 32, 4, 0), (4097, 1, 1, 1), (5, 3, 2, 1), (70_001, 7, 8, 0),
                                        (300_000, 128, 8, 1), (33, 0, 3, 1), (33, 0, 2, 0)])
def test_combination_against_fp64(qk, n, k, nw, acc):
    # W_o = (acc ? W_o : 0) + sum_j C_oj V_j, the update half of the block
    # Gram-Schmidt; FP32 sums in ascending j, held to their rounding bound
    cudart = _cudart()
    rng = np.random.default_rng(n + k + nw)
    V = (rng.standard_normal((k, n)) + 1j * rng.standard_normal((k, n))).astype(np.complex64)
    W0 = (rng.standard_normal((nw, n)) + 1j * rng.standard_normal((nw, n))).astype(np.complex64)
    C = rng.standard_normal((nw, k)) + 1j * rng.standard_normal((nw, k))
    dv = [_dev(cudart, V[j]) for j in range(k)]
    dw = [_dev(cudart, W0[o]) for o in range(nw)]
    try:
        va = (ctypes.c_void_p * max(1, k))(*[p.value for p in dv])
        wa = (ctypes.c_void_p * nw)(*[p.value for p in dw])
        cf = np.ascontiguousarray(C).view(np.float64)
        rc = qk.lib().qkrylov_vector_mcombine_device_f32(va, k, cf.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                                         wa, nw, n, acc, None)
        assert rc == 0, qk.lib().qkrylov_last_error()
        C32 = C.astype(np.complex64).astype(np.complex128)
        ref = C32 @ V.astype(np.complex128) + (W0.astype(np.complex128) if acc else 0)
        scale = np.abs(C32) @ np.abs(V).astype(np.float64) + (np.abs(W0) if acc else 0) + 1e-30
        got = np.empty((nw, n), dtype=np.complex64)
        for o in range(nw):
            assert cudart.cudaMemcpy(got[o].ctypes.data_as(ctypes.c_void_p), dw[o], got[o].nbytes, 2) == 0
        err = np.abs(got - ref) / scale
        assert err.max() <= 4 * (k + 2) * 2.0 ** -24, err.max()
    finally:
        for p in dv + dw:
            cudart.cudaFree(p)


def test_projection_kernel_arguments(qk):
    out = np.zeros(2)
    va = (ctypes.c_void_p * 1)(16)
    dp = out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    L = qk.lib()
    # rejected before any device access
    assert L.qkrylov_vector_mdot_device_f32(va, 129, va, 1, 8, 1, dp, None) == qk.ERROR_INVALID_ARG  # k > 128
    assert L.qkrylov_vector_mdot_device_f32(va, 1, va, 5, 8, 1, dp, None) == qk.ERROR_INVALID_ARG    # nw > 4
    assert L.qkrylov_vector_mdot_device_f32(va, 1, va, 1, 8, 3, dp, None) == qk.ERROR_INVALID_ARG    # method
    v8 = (ctypes.c_void_p * 1)(24)  # off the 16-byte grid: the tensor-core kernel refuses it
    assert L.qkrylov_vector_mdot_device_f32(v8, 1, va, 1, 8, 1, dp, None) == qk.ERROR_INVALID_ARG
    assert L.qkrylov_vector_mdot_device_f32(va, 1, v8, 1, 8, 1, dp, None) == qk.ERROR_INVALID_ARG
    assert L.qkrylov_set_projection_kernel(7) == qk.ERROR_INVALID_ARG
    cp = np.zeros(2 * 1025).ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    assert L.qkrylov_vector_mcombine_device_f32(va, 1, cp, va, 9, 8, 0, None) == qk.ERROR_INVALID_ARG   # nw > 8
    assert L.qkrylov_vector_mcombine_device_f32(va, 129, cp, va, 8, 8, 0, None) == qk.ERROR_INVALID_ARG  # k nw > 1024
    assert L.qkrylov_vector_mcombine_device_f32(va, 1, None, va, 1, 8, 0, None) == qk.ERROR_INVALID_ARG  # no coefficients
    v4 = (ctypes.c_void_p * 1)(20)  # off the 8-byte grid of complex FP32 elements
    assert L.qkrylov_vector_mdot_device_f32(v4, 1, va, 1, 8, 2, dp, None) == qk.ERROR_INVALID_ARG
    assert L.qkrylov_vector_mdot_device_f32(va, 1, v4, 1, 8, 0, dp, None) == qk.ERROR_INVALID_ARG
    assert L.qkrylov_vector_mcombine_device_f32(v4, 1, cp, va, 1, 8, 0, None) == qk.ERROR_INVALID_ARG
    assert L.qkrylov_vector_mcombine_device_f32(va, 1, cp, v4, 1, 8, 0, None) == qk.ERROR_INVALID_ARG


@pytest.mark.parametrize("kernel", ["tensor", "cuda", "fast"])
@pytest.mark.parametrize("model", ["heis", "hub"])
def test_mixed_davidson_with_each_projection_kernel(qk, model, kernel):
    # the mixed Davidson with its projections on the tensor cores, the
    # compensated kernel or the run-summed one (the default): eigenvalues agree
    # with the FP64 form's
    if model == "heis":
        b, s, o = make_model(qk, M.SPIN, 14, M.sector(sz2=0), M.heisenberg_terms(14, True, Jz=0.9))
    else:
        b, s, o = make_model(qk, M.HUBBARD, 8, M.sector(nup=4, ndn=4), M.hubbard_terms(8, True))
    H = qk.MatrixFreeHamiltonian(b, s, o)
    r64 = qk.davidson_lowest_ex(H, n_eig=2, max_subspace=24, tol=1e-8, mixed=False)
    qk.set_projection_kernel(kernel)
    try:
        r32 = qk.davidson_lowest_ex(H, n_eig=2, max_subspace=24, tol=1e-5, mixed=True)
    finally:
        qk.set_projection_kernel("fast")  # the default
    assert np.all(np.asarray(r32.residuals) <= 3e-5), r32.residuals
    np.testing.assert_allclose(r32.eigenvalues, r64.eigenvalues, rtol=0, atol=1e-8)
