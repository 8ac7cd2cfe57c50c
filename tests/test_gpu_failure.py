"""Failure detection without a GPU fault: an allocation that fails as
cudaMalloc does on an exhausted GPU (injected on the host, at every point of a
Hamiltonian's creation and of a solve) must give NULL or QKRYLOV_ERROR_CUDA
with a message, leak no device memory and leave the context usable; and a
bounded device wait that runs out (an mbarrier nothing completes, no copy in
flight) must be counted and reported as QKRYLOV_ERROR_DEVICE_TIMEOUT.  The
reference turns every exception into a status code at its C boundary
(src/c_api.cpp:57-62); these are the failures a GPU adds."""
import ctypes

import numpy as np
import pytest

import models as M
from conftest import make_model

pytestmark = pytest.mark.gpu


def _handles(qk, b, s, o):
    return b._h, s._h, o._h


@pytest.fixture
def no_injection(qk):
    yield
    qk.lib().qkrylov_debug_inject_alloc_failure(-1)


def test_alloc_failure_at_hamiltonian_creation(qk, no_injection):
    L = qk.lib()
    L.qkrylov_hamiltonian_create.restype = ctypes.c_void_p
    b, s, o = make_model(qk, *M.heisenberg(14, True, 0))
    H0 = qk.MatrixFreeHamiltonian(b, s, o)  # the basis' device tables exist from here on
    e0 = qk.lanczos_ground_state(H0, maxiter=300, tol=1e-12).energy
    base = L.qkrylov_debug_live_allocations()
    created = False
    for n in range(0, 200):
        L.qkrylov_debug_inject_alloc_failure(n)
        h = L.qkrylov_hamiltonian_create(*_handles(qk, b, s, o))
        L.qkrylov_debug_inject_alloc_failure(-1)
        if not h:
            assert b"injected" in L.qkrylov_last_error()
            assert L.qkrylov_debug_live_allocations() == base, n
            continue
        L.qkrylov_hamiltonian_destroy(ctypes.c_void_p(h))
        assert L.qkrylov_debug_live_allocations() == base
        created = True
        break
    assert created and n > 3  # creation made several allocations, each one failed once
    # the context is still usable
    assert abs(qk.lanczos_ground_state(H0, maxiter=300, tol=1e-12).energy - e0) <= 1e-12 * abs(e0)


@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
def test_alloc_failure_in_a_solve(qk, no_injection, mixed):
    L = qk.lib()
    b, s, o = make_model(qk, *M.heisenberg(16, True, 0))
    H = qk.MatrixFreeHamiltonian(b, s, o)
    e0 = qk.lanczos_ground_state(H, maxiter=300, tol=1e-12, mixed=mixed).energy
    H.workspace_bytes(release=True)
    base = L.qkrylov_debug_live_allocations()
    fails = 0
    for n in range(0, 60):
        L.qkrylov_debug_inject_alloc_failure(n)
        try:
            r = qk.lanczos_ground_state(H, maxiter=300, tol=1e-12, mixed=mixed)
            ok = True
        except qk.QKrylovError as e:
            ok = False
            assert e.code == qk.ERROR_CUDA and "injected" in str(e), e
        L.qkrylov_debug_inject_alloc_failure(-1)
        H.workspace_bytes(release=True)
        assert L.qkrylov_debug_live_allocations() == base, n
        if ok:
            assert abs(r.energy - e0) <= 1e-10 * abs(e0)
            break
        fails += 1
    assert fails >= 2
    assert abs(qk.lanczos_ground_state(H, maxiter=300, tol=1e-12, mixed=mixed).energy - e0) <= 1e-10 * abs(e0)


def test_device_wait_give_up_is_reported(qk):
    L = qk.lib()
    c0 = qk.device_wait_timeouts()
    assert L.qkrylov_debug_device_wait_probe(1_000_000) == qk.SUCCESS  # 1 ms, nothing completes the barrier
    cnt = ctypes.c_uint32()
    assert L.qkrylov_device_wait_timeouts(ctypes.byref(cnt)) == qk.ERROR_DEVICE_TIMEOUT
    assert cnt.value == c0 + 1
    assert L.qkrylov_debug_device_wait_probe(0) == qk.ERROR_INVALID_ARG
    # the GPU is still usable and a later SpMV is exact
    b, s, o = make_model(qk, *M.heisenberg(12, True, 0))
    H = qk.MatrixFreeHamiltonian(b, s, o)
    x = np.ones(H.dimension, dtype=complex)
    assert np.array_equal(H.apply(x), 3.0 * x)  # H 1 = (L/4) 1 on the periodic chain
    assert qk.device_wait_timeouts() == c0 + 1
