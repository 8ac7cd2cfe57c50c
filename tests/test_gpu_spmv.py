"""GPU y = Hx against the reference: generated matrix entries bit-exact
(indices, order, values), y and the diagonal against the golden fixtures and
the oracle, FP32 kernel within its tolerance, and full-size properties."""
import ctypes

import numpy as np
import pytest

import models as M
from conftest import golden_names, golden_terms, load_golden, make_model
from oracle_ctypes import OHam

pytestmark = pytest.mark.gpu

# FP64 tolerance: the kernel sums a row's diagonal entries first and the
# off-diagonal ones in term order (the reference sums the CSR row in order);
# the difference is rounding only.
RTOL64 = 1e-13
# FP32 kernel: x rounded to FP32 and FP32 accumulation over ~10-100 entries.
RTOL32 = 2e-6


def gpu_ham(qk, g):
    basis, site, ops = make_model(qk, g["model"], g["nsites"], g["sector"], golden_terms(g))
    return qk.MatrixFreeHamiltonian(basis, site, ops)


def apply32(qk, H, x):
    """FP32 kernel through the device-pointer ABI (vectors staged with the CUDA runtime)."""
    cudart = _cudart()
    n = H.dimension
    xs = np.ascontiguousarray(x, dtype=np.complex64)
    y = np.zeros(n, dtype=np.complex64)
    dx, dy = ctypes.c_void_p(), ctypes.c_void_p()
    assert cudart.cudaMalloc(ctypes.byref(dx), max(8, 8 * n)) == 0
    assert cudart.cudaMalloc(ctypes.byref(dy), max(8, 8 * n)) == 0
    try:
        assert cudart.cudaMemcpy(dx, xs.ctypes.data_as(ctypes.c_void_p), 8 * n, 1) == 0
        H.apply_device(dx.value, dy.value, None, fp32=True)
        assert cudart.cudaDeviceSynchronize() == 0
        assert cudart.cudaMemcpy(y.ctypes.data_as(ctypes.c_void_p), dy, 8 * n, 2) == 0
    finally:
        cudart.cudaFree(dx)
        cudart.cudaFree(dy)
    return y


_CUDART = None


def _cudart():
    global _CUDART
    if _CUDART is None:
        import ctypes.util
        for name in ("libcudart.so", "libcudart.so.13", "libcudart.so.12", ctypes.util.find_library("cudart")):
            try:
                if name:
                    _CUDART = ctypes.CDLL(name)
                    break
            except OSError:
                continue
        if _CUDART is None:
            import glob
            cands = glob.glob("/usr/local/cuda/lib64/libcudart.so*") + glob.glob("/usr/local/cuda/targets/*/lib/libcudart.so*")
            _CUDART = ctypes.CDLL(cands[0])
        _CUDART.cudaMalloc.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_size_t]
        _CUDART.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
        _CUDART.cudaFree.argtypes = [ctypes.c_void_p]
    return _CUDART


@pytest.mark.parametrize("name", golden_names())
def test_entries_bit_exact(qk, name):
    """Every generated (row, column, value) in the reference's order
    (src/hamiltonian/matrix_free_hamiltonian.cpp:45-92)."""
    g = load_golden(name)
    if "csr_ro" not in g:
        pytest.skip("fixture without CSR")
    H = gpu_ham(qk, g)
    ro, cols, vals = H.entries()
    assert np.array_equal(ro.astype(np.int64), g["csr_ro"].astype(np.int64))
    assert np.array_equal(cols.astype(np.int64), g["csr_cols"].astype(np.int64))
    np.testing.assert_allclose(vals, g["csr_vals"], rtol=0, atol=1e-15)


@pytest.mark.parametrize("mode", [0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10],
                         ids=["auto", "generic", "fast", "fast-staged", "fast-rows4", "fast-rows4-staged", "fast-rows4-wide",
                              "tile1", "tile2", "tile4", "class"])
@pytest.mark.parametrize("name", golden_names())
def test_apply_and_diagonal(qk, name, mode):
    g = load_golden(name)
    H = gpu_ham(qk, g)
    H.select_kernel(mode=mode)
    assert H.dimension == int(g["dim"])
    np.testing.assert_array_equal(H.diagonal(), g["diag"].real)  # summed in term order: bit-exact
    if "x" in g:
        y = H.apply(g["x"])
        scale = np.abs(g["y"]).max()
        assert np.abs(y - g["y"]).max() <= RTOL64 * scale
        y32 = apply32(qk, H, g["x"])
        assert np.abs(y32 - g["y"]).max() <= RTOL32 * scale * 10


@pytest.mark.parametrize("mode", [3, 5, 7, 10], ids=["fast-staged", "fast-rows4-staged", "tile1", "class"])
def test_staged_variant_after_a_smaller_hamiltonian(qk, mode):
    # a kernel's shared-memory limit is set per kernel and device, not per
    # Hamiltonian: building a smaller model (a smaller staged slice) after a
    # larger one must not make the larger one's staged launches fail
    big = qk.MatrixFreeHamiltonian(*make_model(qk, *M.heisenberg(20, True, 0)))
    big.select_kernel(mode=mode)
    rng = np.random.default_rng(5)
    x = rng.standard_normal(big.dimension) + 1j * rng.standard_normal(big.dimension)
    y0 = big.apply(x)
    small = qk.MatrixFreeHamiltonian(*make_model(qk, *M.heisenberg(4, True, 0)))
    small.apply(np.ones(small.dimension, dtype=np.complex128))
    y1 = big.apply(x)
    np.testing.assert_array_equal(y1, y0)
    big.select_kernel(mode=1)  # the generic kernel as the reference
    np.testing.assert_allclose(y1, big.apply(x), rtol=0, atol=RTOL64 * np.abs(y1).max())


def test_fast_kernel_is_used_where_eligible(qk):
    for m in (M.heisenberg(16, True, 0), M.hubbard(8, True, 4, 4), (M.SPIN, 12, M.sector(), M.xyz_field_terms(12, True)),
              (M.FERMION, 14, M.sector(n=5), M.fermion_chain_terms(14, True))):
        b, s, o = make_model(qk, *m)
        H = qk.MatrixFreeHamiltonian(b, s, o)
        assert H.select_kernel(False), m[:3]
        assert not H.select_kernel(True)


@pytest.mark.parametrize("model,N,sector,terms", [
    (M.SPIN, 20, M.sector(sz2=0), M.heisenberg_terms(20, True)),
    (M.SPIN, 18, M.sector(sz2=2), M.heisenberg_terms(18, False, Jz=0.7)),
    (M.SPIN, 12, M.sector(), M.xyz_field_terms(12, True)),
    (M.FERMION, 16, M.sector(n=6), M.fermion_chain_terms(16, True)),
    (M.HUBBARD, 8, M.sector(nup=4, ndn=4), M.hubbard_terms(8, True)),
    (M.HUBBARD, 7, M.sector(nup=3), M.hubbard_terms(7, False)),
    (M.TJ, 8, M.sector(nup=3, ndn=3), M.tj_terms(8, True)),
])
def test_apply_against_oracle(qk, oracle, model, N, sector, terms):
    basis, site, ops = make_model(qk, model, N, sector, terms)
    H = qk.MatrixFreeHamiltonian(basis, site, ops)
    o = OHam(oracle, model, N, sector, terms)
    assert H.dimension == o.dim
    rng = np.random.default_rng(7)
    x = rng.normal(size=o.dim) + 1j * rng.normal(size=o.dim)
    yo = o.apply(x)
    waits0 = qk.device_wait_timeouts()
    for mode in (0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10):
        H.select_kernel(mode=mode)
        y = H.apply(x)
        assert np.abs(y - yo).max() <= RTOL64 * np.abs(yo).max()
        y32 = apply32(qk, H, x)
        assert np.abs(y32 - yo).max() <= RTOL32 * 10 * np.abs(yo).max()
    # the staged kernels' bounded waits for their asynchronous copies never gave up
    assert qk.device_wait_timeouts() == waits0


def test_edge_cases(qk):
    # empty sector (odd 2Sz on an even chain): dimension 0, calls succeed
    basis, site, ops = make_model(qk, M.SPIN, 6, M.sector(sz2=1), M.heisenberg_terms(6, True))
    H = qk.MatrixFreeHamiltonian(basis, site, ops)
    assert H.dimension == 0
    assert H.apply(np.zeros(0, dtype=complex)).shape == (0,)
    # one site
    basis, site, ops = make_model(qk, M.SPIN, 1, M.sector(), [(0.7, [("Sz", 0)]), (0.2, [("Sx", 0)])])
    H = qk.MatrixFreeHamiltonian(basis, site, ops)
    y = H.apply(np.array([1.0, 0.0], dtype=complex))
    np.testing.assert_allclose(y, [-0.35, 0.1], atol=1e-15)
    # a site beyond the chain behaves as an always-down spin (bits above N are 0):
    # Sz(5) on 4 sites contributes -0.5 to every diagonal entry; Sp(5) leaves the basis
    basis, site, ops = make_model(qk, M.SPIN, 4, M.sector(), [(1.0, [("Sz", 5)]), (1.0, [("Sp", 5)])])
    H = qk.MatrixFreeHamiltonian(basis, site, ops)
    np.testing.assert_array_equal(H.diagonal(), -0.5 * np.ones(16))
    # unknown operator / site outside the 64-bit state: creation fails loudly
    basis, site, ops = make_model(qk, M.SPIN, 4, M.sector(), [(1.0, [("Sq", 0)])])
    with pytest.raises(ValueError, match="Unknown spin operator"):
        qk.MatrixFreeHamiltonian(basis, site, ops)
    basis, site, ops = make_model(qk, M.HUBBARD, 4, M.sector(), [(1.0, [("CUp", 40)])])
    with pytest.raises(ValueError, match="out of range"):
        qk.MatrixFreeHamiltonian(basis, site, ops)
    # wrong vector length
    basis, site, ops = make_model(qk, M.SPIN, 4, M.sector(), M.heisenberg_terms(4, False))
    H = qk.MatrixFreeHamiltonian(basis, site, ops)
    with pytest.raises(ValueError):
        H.apply(np.zeros(3, dtype=complex))


@pytest.mark.parametrize("m", [M.heisenberg(16, True, 0), M.hubbard(6, True, 3, 2)])
def test_apply_torch_cuda_tensor_zero_copy(qk, m):
    """H.apply on a torch CUDA tensor (complex128 and complex64) runs on the
    device pointers in reference order and matches the host path."""
    torch = pytest.importorskip("torch")
    b, s, o = make_model(qk, *m)
    H = qk.MatrixFreeHamiltonian(b, s, o)
    rng = np.random.default_rng(4)
    x = rng.normal(size=H.dimension) + 1j * rng.normal(size=H.dimension)
    y = H.apply(x)
    xt = torch.from_numpy(x).to("cuda:0")
    yt = H.apply(xt)
    assert isinstance(yt, torch.Tensor) and yt.is_cuda and yt.dtype == torch.complex128
    np.testing.assert_allclose(yt.cpu().numpy(), y, rtol=0, atol=RTOL64 * np.abs(y).max())
    y32 = H.apply(xt.to(torch.complex64))
    assert y32.dtype == torch.complex64
    np.testing.assert_allclose(y32.cpu().numpy(), y, rtol=0, atol=RTOL32 * np.abs(y).max() * 4)
    with pytest.raises(ValueError):
        H.apply(xt[:-1])


def test_reference_c_api_float_entry_points(qk):
    """tests/test_c_api.cpp:92-149 through the float ABI."""
    L = qk.lib()
    sec = L.qkrylov_sector_create()
    L.qkrylov_sector_set_sz(sec, 0)
    basis = L.qkrylov_spinhalf_basis_create(4, sec)
    assert L.qkrylov_basis_dimension(basis) == 6
    site = L.qkrylov_spinhalf_site_create()
    op = L.qkrylov_opsum_create()
    for i in range(3):
        assert L.qkrylov_opsum_add_term_2body(op, 1.0, 0.0, b"Sz", i, b"Sz", i + 1) == 0
        assert L.qkrylov_opsum_add_term_2body(op, 0.5, 0.0, b"Sp", i, b"Sm", i + 1) == 0
        assert L.qkrylov_opsum_add_term_2body(op, 0.5, 0.0, b"Sm", i, b"Sp", i + 1) == 0
    H = L.qkrylov_hamiltonian_create(basis, site, op)
    assert H
    dim = 6
    xr, xi = np.ones(dim, np.float32), np.zeros(dim, np.float32)
    yr, yi = np.zeros(dim, np.float32), np.zeros(dim, np.float32)
    fp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    assert L.qkrylov_hamiltonian_apply(H, fp(xr), fp(xi), fp(yr), fp(yi)) == 0
    xc = np.zeros(2 * dim, np.float32)
    xc[0::2] = 1
    yc = np.zeros(2 * dim, np.float32)
    assert L.qkrylov_hamiltonian_apply_complex(H, fp(xc), fp(yc)) == 0
    np.testing.assert_array_equal(yc[0::2], yr)
    g = dict(np.load(__import__("conftest").GOLDEN + "/capi_heis4.npz"))
    np.testing.assert_allclose(yc, g["y"], atol=1e-6)
    d = np.zeros(dim, np.float32)
    assert L.qkrylov_hamiltonian_diagonal(H, fp(d)) == 0
    r = qk.LanczosResultC()
    psi = np.zeros(2 * dim, np.float32)
    assert L.qkrylov_lanczos_ground_state_complex(H, 200, 1e-12, ctypes.byref(r), fp(psi)) == 0
    assert abs(r.energy + 1.6160254038) < 1e-5
    assert abs(float(np.sum(psi.astype(np.float64) ** 2)) - 1.0) < 1e-4
    ev = np.zeros(2, np.float32)
    evec = np.zeros(4 * dim, np.float32)
    info = qk.DavidsonResultC()
    assert L.qkrylov_davidson_lowest_complex(H, 2, 20, 1e-6, fp(ev), fp(evec), ctypes.byref(info)) == 0
    assert info.converged == 1 and abs(ev[0] - r.energy) < 1e-4 and ev[0] <= ev[1]
    for k in range(2):
        v = evec[2 * k * dim:2 * (k + 1) * dim]
        hv = np.zeros_like(v)
        assert L.qkrylov_hamiltonian_apply_complex(H, fp(v), fp(hv)) == 0
        assert np.abs(hv - ev[k] * v).max() < 1e-3
    a, b, nrm = np.zeros(20, np.float32), np.zeros(20, np.float32), np.zeros(1, np.float32)
    nc = ctypes.c_int()
    assert L.qkrylov_continued_fraction_coeffs_complex(H, fp(psi), 20, fp(a), fp(b), fp(nrm), ctypes.byref(nc)) == 0
    assert nc.value > 0 and abs(nrm[0] - 1) < 1e-3
    assert L.qkrylov_evaluate_spectral_function(fp(a), fp(b), nc.value, nrm[0], 0.5, r.energy, 0.1) > 0
    fr = qk.FTLMResultC()
    assert L.qkrylov_ftlm(H, 1.0, 10, 20, ctypes.byref(fr)) == 0
    assert fr.partition_function > 0
    np.testing.assert_allclose([fr.partition_function, fr.internal_energy, fr.specific_heat], g["ftlm"][1:], rtol=1e-4)
    for f, hnd in ((L.qkrylov_hamiltonian_destroy, H), (L.qkrylov_opsum_destroy, op), (L.qkrylov_site_destroy, site),
                   (L.qkrylov_basis_destroy, basis), (L.qkrylov_sector_destroy, sec)):
        f(hnd)


def test_full_size_heisenberg_L28_properties(qk, oracle):
    """Heisenberg L=28 periodic chain, Sz=0, at full size (dim 40,116,600): sampled rows against
    the oracle's CSR rows, Hermiticity, and H 1 = (L/4) 1 (the Sz=0 member of
    the ferromagnetic multiplet)."""
    L = 28
    basis, site, ops = make_model(qk, M.SPIN, L, M.sector(sz2=0), M.heisenberg_terms(L, True))
    H = qk.MatrixFreeHamiltonian(basis, site, ops)
    n = H.dimension
    assert n == 40116600
    ones = np.ones(n, dtype=np.complex128)
    y = H.apply(ones)
    assert np.array_equal(y, (L / 4) * ones)
    rng = np.random.default_rng(3)
    x = (rng.standard_normal(n) + 1j * rng.standard_normal(n))
    z = (rng.standard_normal(n) + 1j * rng.standard_normal(n))
    waits0 = qk.device_wait_timeouts()
    hx, hz = H.apply(x), H.apply(z)
    lhs, rhs = np.vdot(z, hx), np.vdot(hz, x)
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)
    # every fast variant (the tiled ones included) gives the same y at full size
    for mode in (4, 7, 8, 9, 10):
        H.select_kernel(mode=mode)
        assert np.abs(H.apply(x) - hx).max() <= RTOL64 * np.abs(hx).max(), mode
        assert np.abs(apply32(qk, H, x) - hx).max() <= RTOL32 * 10 * np.abs(hx).max(), mode
    H.select_kernel(mode=0)
    assert qk.device_wait_timeouts() == waits0
    # exact rows from the oracle for three row windows (first, middle, last block)
    from oracle_ctypes import Oracle
    import ctypes as c
    lib = oracle.lib
    lib.qko_sample_create.restype = c.c_void_p
    terms = M.heisenberg_terms(L, True)
    cre = np.array([t[0] for t in terms], dtype=np.float64)
    cim = np.zeros_like(cre)
    nf = np.array([len(t[1]) for t in terms], dtype=np.int32)
    fl = [f for t in terms for f in t[1]]
    opsa = (c.c_char_p * len(fl))(*[f[0].encode() for f in fl])
    sites = np.array([f[1] for f in fl], dtype=np.int32)
    sec = np.array(M.sector(sz2=0), dtype=np.int32)
    for row0 in (0, n // 2 - 1500, n - 3000):
        h = lib.qko_sample_create(0, L, sec.ctypes.data_as(c.POINTER(c.c_int)), len(terms),
                                  cre.ctypes.data_as(c.POINTER(c.c_double)), cim.ctypes.data_as(c.POINTER(c.c_double)),
                                  nf.ctypes.data_as(c.POINTER(c.c_int)), opsa, sites.ctypes.data_as(c.POINTER(c.c_int)),
                                  c.c_uint64(row0), c.c_uint64(3000))
        ys = np.zeros(3000, dtype=np.complex128)
        lib.qko_apply(c.c_void_p(h), x.ctypes.data_as(c.POINTER(c.c_double)), ys.ctypes.data_as(c.POINTER(c.c_double)))
        lib.qko_destroy(c.c_void_p(h))
        assert np.abs(hx[row0:row0 + 3000] - ys).max() <= RTOL64 * np.abs(ys).max()


def test_full_size_hubbard_L16_properties(qk):
    """Hubbard L=16 periodic chain, half filling, at full size (dim 165,636,900): Hermiticity and
    particle-hole/total-number checks."""
    Lh = 16
    basis, site, ops = make_model(qk, M.HUBBARD, Lh, M.sector(nup=8, ndn=8), M.hubbard_terms(Lh, True))
    H = qk.MatrixFreeHamiltonian(basis, site, ops)
    n = H.dimension
    assert n == 12870 ** 2
    info = H.info()
    assert info["n_diag"] == 16 and info["diag_mode"] == 0
    rng = np.random.default_rng(5)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    z = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    lhs, rhs = np.vdot(z, H.apply(x)), np.vdot(H.apply(z), x)
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)
    d = H.diagonal()
    assert d.min() == 0.0 and d.max() == 4.0 * 8  # U * number of doubly occupied sites
