"""The C-ABI library loads, exports every symbol include/*.h declares, and its
host-side parts (sectors, bases, OpSums, argument checks) behave like the
reference's C API without a GPU."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

import models as M
from conftest import ROOT, golden_names, golden_terms, load_golden
from oracle_ctypes import OHam


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "**", "*.h"), recursive=True):
        txt = re.sub(r"/\*.*?\*/", "", open(h).read(), flags=re.S)
        names |= set(re.findall(r"\b(qkrylov_[a-z0-9_]+)\s*\(", txt))
    return sorted(names)


def test_every_declared_symbol_is_exported(qk):
    names = declared_functions()
    assert len(names) > 60
    missing = [n for n in names if not hasattr(qk.lib(), n)]
    assert not missing, missing


def test_reference_symbols_all_present(qk):
    # every function of the reference C API (include/qkrylov/c_api.h:30-168)
    ref = """sector_create sector_destroy sector_set_sz sector_set_hubbard_particles sector_set_n sector_set_nb
    sector_get_sz sector_get_hubbard_particles sector_get_n sector_get_nb spinhalf_basis_create fermion_basis_create
    hubbard_basis_create tj_basis_create basis_destroy basis_dimension basis_nsites basis_state basis_index
    basis_contains spinhalf_site_create fermion_site_create hubbard_site_create tj_site_create site_destroy
    opsum_create opsum_destroy opsum_clear opsum_add_term_1body opsum_add_term_2body opsum_add_term_nbody
    hamiltonian_create hamiltonian_destroy hamiltonian_dimension hamiltonian_apply hamiltonian_apply_complex
    hamiltonian_diagonal lanczos_ground_state lanczos_ground_state_complex davidson_lowest_complex
    continued_fraction_coeffs_complex evaluate_spectral_function ftlm""".split()
    for n in ref:
        assert hasattr(qk.lib(), "qkrylov_" + n)


def test_sector_semantics(qk):
    L = qk.lib()
    s = L.qkrylov_sector_create()
    v, a = ctypes.c_int(), ctypes.c_int()
    assert L.qkrylov_sector_get_sz(s, ctypes.byref(v), ctypes.byref(a)) == 0 and a.value == 0
    assert L.qkrylov_sector_set_sz(s, -2) == 0
    L.qkrylov_sector_get_sz(s, ctypes.byref(v), ctypes.byref(a))
    assert (v.value, a.value) == (-2, 1)
    n2 = ctypes.c_int()
    assert L.qkrylov_sector_set_hubbard_particles(s, 3, 4) == 0
    L.qkrylov_sector_get_hubbard_particles(s, ctypes.byref(v), ctypes.byref(n2), ctypes.byref(a))
    assert (v.value, n2.value, a.value) == (3, 4, 1)
    assert L.qkrylov_sector_set_nb(s, 2) == 0
    L.qkrylov_sector_get_nb(s, ctypes.byref(v), ctypes.byref(a))
    assert (v.value, a.value) == (2, 1)
    L.qkrylov_sector_destroy(s)
    # NULL handles: -1, 0 or NULL like the reference (c_api.cpp:69-78, 209-257)
    assert L.qkrylov_sector_set_sz(None, 0) == qk.ERROR_INVALID_ARG
    assert L.qkrylov_sector_get_n(None, None, None) == qk.ERROR_INVALID_ARG
    assert L.qkrylov_basis_dimension(None) == 0
    assert L.qkrylov_basis_index(None, 3) == -1
    assert L.qkrylov_basis_contains(None, 3) == 0
    assert L.qkrylov_hamiltonian_create(None, None, None) is None
    assert L.qkrylov_opsum_add_term_1body(None, 1.0, 0.0, b"Sz", 0) == qk.ERROR_INVALID_ARG
    assert L.qkrylov_opsum_add_term_nbody(L.qkrylov_opsum_create(), 1.0, 0.0, 0, None, None) == qk.ERROR_INVALID_ARG
    r = qk.LanczosResultC()
    assert L.qkrylov_lanczos_ground_state(None, 10, 1e-8, ctypes.byref(r)) == qk.ERROR_INVALID_ARG
    assert L.qkrylov_evaluate_spectral_function(None, None, 0, 1.0, 0.0, 0.0, 0.1) == 0.0
    # additions: invalid arguments are rejected before any device work
    held = ctypes.c_uint64()
    assert L.qkrylov_hamiltonian_workspace(None, 0, ctypes.byref(held)) == qk.ERROR_INVALID_ARG
    assert L.qkrylov_hamiltonian_workspace(None, 1, None) == qk.ERROR_INVALID_ARG
    assert L.qkrylov_device_wait_timeouts(None) == qk.ERROR_INVALID_ARG
    assert L.qkrylov_hamiltonian_benchmark_apply(None, 1, 3, None) == qk.ERROR_INVALID_ARG
    assert L.qkrylov_hamiltonian_tuning(None, 1, None, None) == qk.ERROR_INVALID_ARG
    vals, n_out = np.zeros(4), ctypes.c_int()
    dv = vals.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    assert L.qkrylov_lanczos_ritz_values(None, 10, 0, 1, 4, dv, ctypes.byref(n_out), None) == qk.ERROR_INVALID_ARG
    out = np.zeros(2)
    ptrs = (ctypes.c_void_p * 1)(16)
    dp = out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    assert L.qkrylov_vector_mdot_device_f32(None, 1, ptrs, 1, 8, 0, dp, None) == qk.ERROR_INVALID_ARG
    assert L.qkrylov_vector_mdot_device_f32(ptrs, 0, ptrs, 1, 8, 0, dp, None) == qk.ERROR_INVALID_ARG
    # device pointers off the grid of whole complex elements: refused before any launch
    res = (ctypes.c_double * 2)()
    assert L.qkrylov_vector_dot_device_f64(ctypes.c_void_p(24), ctypes.c_void_p(32), 4, res, None) == qk.ERROR_INVALID_ARG
    assert L.qkrylov_vector_dot_device_f32(ctypes.c_void_p(16), ctypes.c_void_p(20), 4, res, None) == qk.ERROR_INVALID_ARG
    assert L.qkrylov_vector_dot_device_f64_noalloc(ctypes.c_void_p(8), ctypes.c_void_p(16), 4, res, None) == qk.ERROR_INVALID_ARG
    bad = (ctypes.c_void_p * 1)(12)
    assert L.qkrylov_vector_mcombine_device_f32(bad, 1, dp, ptrs, 1, 8, 0, None) == qk.ERROR_INVALID_ARG
    assert L.qkrylov_set_projection_kernel(3) == qk.ERROR_INVALID_ARG


@pytest.mark.parametrize("name", golden_names())
def test_basis_bit_exact_against_reference(qk, name):
    """state(i) / index(s) / contains(s) of the combinatorial tables equal the
    reference's enumerate-and-hash basis (src/basis/*.cpp) state for state."""
    g = load_golden(name)
    from conftest import make_model
    basis, _, _ = make_model(qk, g["model"], g["nsites"], g["sector"], [])
    assert basis.size == int(g["dim"])
    assert basis.nsites == int(g["nsites"])
    st = g["states"]
    got = np.array([basis.state(i) for i in range(basis.size)], dtype=np.uint64)
    assert np.array_equal(got, st)
    for i in range(0, len(st), max(1, len(st) // 300)):
        assert basis.index(int(st[i])) == i
        assert basis.contains(int(st[i]))
    nbits = int(g["nsites"]) * (2 if int(g["model"]) >= 2 else 1)
    present = set(int(s) for s in st)
    rng = np.random.default_rng(1)
    for s in rng.integers(0, 1 << nbits, size=200):
        s = int(s)
        assert basis.contains(s) == (s in present)
        if s not in present:
            assert basis.index(s) == -1
    assert basis.index(1 << nbits) == -1


@pytest.mark.parametrize("model,N,sector", [
    (M.SPIN, 20, M.sector(sz2=0)), (M.SPIN, 19, M.sector(sz2=-3)), (M.SPIN, 13, M.sector()),
    (M.FERMION, 18, M.sector(n=5)), (M.HUBBARD, 8, M.sector(nup=4, ndn=4)), (M.HUBBARD, 7, M.sector(ndn=2)),
    (M.TJ, 8, M.sector(nup=3, ndn=3)), (M.SPIN, 10, M.sector(sz2=1)), (M.SPIN, 1, M.sector(sz2=1)),
])
def test_larger_bases_against_oracle(qk, oracle, model, N, sector):
    from conftest import make_model
    basis, _, _ = make_model(qk, model, N, sector, [])
    o = OHam(oracle, model, N, sector, [])
    assert basis.size == o.dim
    st = o.states()
    idx = np.unique(np.linspace(0, max(0, o.dim - 1), num=min(o.dim, 2000)).astype(np.int64)) if o.dim else []
    for i in idx:
        assert basis.state(int(i)) == int(st[i])
        assert basis.index(int(st[i])) == int(i)


def test_basis_errors_return_null(qk):
    L = qk.lib()
    assert L.qkrylov_spinhalf_basis_create(0, None) is None
    assert L.qkrylov_spinhalf_basis_create(64, None) is None
    assert L.qkrylov_hubbard_basis_create(32, None) is None
    assert b"N must satisfy" in L.qkrylov_last_error()
    b = L.qkrylov_spinhalf_basis_create(3, None)
    assert L.qkrylov_basis_state(b, 8) == 0  # out of range -> 0 (c_api.cpp:231-238)
    L.qkrylov_basis_destroy(b)


def test_opsum_python_sugar(qk):
    os_ = qk.OpSum()
    os_ += 1.0 * qk.Sz(0) * qk.Sz(1) + 0.5 * (qk.Sp(0) * qk.Sm(1)) + 0.5 * qk.Sm(0) * qk.Sp(1)
    assert len(os_) == 3
    assert os_.terms[1] == (0.5 + 0j, [("Sp", 0), ("Sm", 1)])
    with pytest.raises(ValueError):
        os_ += (1.0, "Sz")


def test_spectral_grid_equals_pointwise(qk):
    """The frequency grid (evaluated in parallel for large grids) gives, value for
    value, the single-frequency continued fraction (dynamics.cpp:61-89)."""
    rng = np.random.default_rng(5)

    class R:
        pass
    r = R()
    r.alphas, r.betas, r.norm_phi0 = rng.normal(size=120), np.abs(rng.normal(size=120)), 0.8
    om = np.linspace(-1.0, 5.0, 1200)
    grid = qk.evaluate_spectral_function(r, om, -3.0, 0.07)
    point = np.array([qk.evaluate_spectral_function(r, float(w), -3.0, 0.07) for w in om[::37]])
    np.testing.assert_array_equal(grid[::37], point)
    assert np.all(grid >= 0)
