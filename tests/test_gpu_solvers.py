"""GPU solvers against the reference: Lanczos E0 within 1e-10 relative,
Davidson eigenvalues, continued-fraction coefficients and S(omega), FTLM
tridiagonals and Z/E/Cv within 1e-8, and the mixed form's |dE0| against FP64."""
import numpy as np
import pytest

import models as M
from conftest import golden_names, golden_terms, load_golden, make_model
from oracle_ctypes import OHam, spectral

pytestmark = pytest.mark.gpu

E0_RTOL = 1e-10    # the bar for E0 against the reference's FP64 Lanczos (relative)
DYN_RTOL = 1e-8    # S(omega), FTLM Z/E/Cv


def gpu_ham(qk, g):
    basis, site, ops = make_model(qk, g["model"], g["nsites"], g["sector"], golden_terms(g))
    return qk.MatrixFreeHamiltonian(basis, site, ops)


@pytest.mark.parametrize("name", golden_names())
def test_lanczos_energy(qk, name):
    g = load_golden(name)
    H = gpu_ham(qk, g)
    r = qk.lanczos_ground_state(H, maxiter=300, tol=1e-12)
    e_ref = float(g["lanczos_E0"])
    assert abs(r.energy - e_ref) <= E0_RTOL * max(1.0, abs(e_ref))
    assert r.converged
    assert abs(r.iterations - int(g["lanczos_iters"])) <= 3
    v = r.eigenvector
    assert abs(np.linalg.norm(v) - 1) < 1e-12
    # |dE| < tol stops the iteration with a residual of order sqrt(tol);
    # the reference's own Ritz test bounds it by 1e-5 (tests/test_lanczos_ritz.cpp:52-55)
    res = np.linalg.norm(H.apply(v) - r.energy * v)
    assert res < 1e-5


def test_heisenberg_L16_obc_lanczos(qk):
    """Heisenberg L=16 open chain, Sz=0, tol 1e-12, <=300 iterations; the
    reference gives E0 = -6.911737145574688 (golden heis_L16_obc_sz0)."""
    g = load_golden("heis_L16_obc_sz0")
    H = gpu_ham(qk, g)
    r = qk.lanczos_ground_state(H, maxiter=300, tol=1e-12)
    assert abs(r.energy - float(g["lanczos_E0"])) <= E0_RTOL * abs(float(g["lanczos_E0"]))
    assert abs(r.energy - (-6.911737145574688)) < 1e-10 * 6.92


@pytest.mark.parametrize("name", golden_names())
def test_davidson(qk, name):
    g = load_golden(name)
    H = gpu_ham(qk, g)
    k = len(g["davidson_evals"])
    r = qk.davidson_lowest(H, n_eig=k, max_subspace=20, tol=1e-8)
    if bool(g["davidson_conv"]):
        assert r.converged
        np.testing.assert_allclose(r.eigenvalues, g["davidson_evals"], rtol=1e-8, atol=1e-8)
        for lam, v in zip(r.eigenvalues, r.eigenvectors):
            assert np.linalg.norm(H.apply(v) - lam * v) <= 1e-6


@pytest.mark.parametrize("name", [n for n in golden_names() if n != "heis_L16_obc_sz0"])
def test_continued_fraction(qk, name):
    g = load_golden(name)
    H = gpu_ham(qk, g)
    r = qk.continued_fraction_coeffs(H, g["cf_phi0"], len(g["cf_alphas"]))
    assert abs(r.norm_phi0 - float(g["cf_norm"])) <= 1e-13 * float(g["cf_norm"])
    k = min(10, len(r.alphas))
    np.testing.assert_allclose(r.alphas[:k], g["cf_alphas"][:k], rtol=1e-9, atol=1e-9)
    np.testing.assert_allclose(r.betas[:k], g["cf_betas"][:k], rtol=1e-9, atol=1e-9)
    # S(omega) from the first 10 coefficients on a grid, same formula as dynamics.cpp:61-89
    om = np.linspace(0.0, 4.0, 41)
    res10 = qk.DynamicsResult(r.alphas[:k], r.betas[:k], r.norm_phi0)
    s_gpu = qk.evaluate_spectral_function(res10, om, E0=-1.0, eta=0.05)
    ref10 = qk.DynamicsResult(g["cf_alphas"][:k], g["cf_betas"][:k], float(g["cf_norm"]))
    s_ref = qk.evaluate_spectral_function(ref10, om, E0=-1.0, eta=0.05)
    np.testing.assert_allclose(s_gpu, s_ref, rtol=DYN_RTOL, atol=DYN_RTOL * np.abs(s_ref).max())


@pytest.mark.parametrize("name", golden_names())
def test_ftlm(qk, name):
    g = load_golden(name)
    H = gpu_ham(qk, g)
    R, Mst = g["ftlm_alphas"].shape
    r = qk.ftlm(H, g["ftlm_betas_T"], n_random=R, n_steps=Mst)
    obs = g["ftlm_obs"]
    np.testing.assert_allclose(r.partition_function, obs[:, 0], rtol=DYN_RTOL)
    np.testing.assert_allclose(r.internal_energy, obs[:, 1], rtol=DYN_RTOL, atol=DYN_RTOL)
    np.testing.assert_allclose(r.specific_heat, obs[:, 2], rtol=DYN_RTOL, atol=DYN_RTOL)
    # shifted evaluation gives the same values after undoing the shift
    s = qk.ftlm(H, g["ftlm_betas_T"], n_random=R, n_steps=Mst, shifted=True)
    np.testing.assert_allclose(s.partition_function * np.exp(s.log_shift), obs[:, 0], rtol=DYN_RTOL)
    np.testing.assert_allclose(s.internal_energy, obs[:, 1], rtol=DYN_RTOL, atol=DYN_RTOL)


def test_reference_known_answers(qk):
    # tests/test_lanczos_ritz.cpp: 2 sites, full basis, E0 = -0.75, Ritz residual < 1e-5
    b, s, o = make_model(qk, M.SPIN, 2, M.sector(), M.heisenberg_terms(2, False))
    H = qk.MatrixFreeHamiltonian(b, s, o)
    r = qk.lanczos_ground_state(H)
    assert abs(r.energy + 0.75) < 1e-5
    assert np.abs(H.apply(r.eigenvector) - r.energy * r.eigenvector).max() < 1e-5
    # bindings/julia/test/runtests.jl:122: periodic 4-site chain, full basis, E0 = -2
    b, s, o = make_model(qk, M.SPIN, 4, M.sector(), M.heisenberg_terms(4, True))
    H = qk.MatrixFreeHamiltonian(b, s, o)
    assert abs(qk.lanczos_ground_state(H, maxiter=50, tol=1e-12).energy + 2.0) < 1e-6
    r2 = qk.lanczos_ground_state(H, maxiter=2, tol=1e-15)
    assert not r2.converged and r2.iterations == 2
    # tests/test_ftlm.cpp: H = Sz0 Sz1 on 2 sites, Z > 0, |E| < 1
    b, s, o = make_model(qk, M.SPIN, 2, M.sector(), [(1.0, [("Sz", 0), ("Sz", 1)])])
    f = qk.ftlm(qk.MatrixFreeHamiltonian(b, s, o), 1.0, 100, 10)
    assert f.partition_function > 0 and abs(f.internal_energy) < 1
    # tests/test_dynamics.cpp: S(0.5) >= 0 from phi0 = e_0
    b, s, o = make_model(qk, M.SPIN, 2, M.sector(), M.heisenberg_terms(2, False))
    H = qk.MatrixFreeHamiltonian(b, s, o)
    e0 = qk.lanczos_ground_state(H).energy
    phi0 = np.zeros(4, dtype=complex)
    phi0[0] = 1
    d = qk.continued_fraction_coeffs(H, phi0, 10)
    assert len(d.alphas) > 0 and qk.evaluate_spectral_function(d, 0.5, e0, 0.1) >= 0


@pytest.mark.parametrize("L", [16, 20])
def test_mixed_form_matches_fp64(qk, L):
    """Mixed form: |dE0| <= 1e-10 relative against the FP64 path."""
    b, s, o = make_model(qk, M.SPIN, L, M.sector(sz2=0), M.heisenberg_terms(L, True))
    H = qk.MatrixFreeHamiltonian(b, s, o)
    r64 = qk.lanczos_ground_state(H, maxiter=300, tol=1e-12)
    rm = qk.lanczos_ground_state(H, maxiter=300, tol=1e-12, mixed=True)
    assert abs(rm.energy - r64.energy) <= 1e-10 * abs(r64.energy)
    assert rm.residual < 1e-4
    ov = abs(np.vdot(rm.eigenvector, r64.eigenvector))
    assert ov > 1 - 1e-8


@pytest.mark.parametrize("m", [M.heisenberg(18, True, 0), M.hubbard(8, True, 4, 4),
                               (M.FERMION, 16, M.sector(n=6), M.fermion_chain_terms(16, True))])
def test_mixed_device_engine_matches_host_driven(qk, m):
    """The device-resident mixed Lanczos (graph-replayed steps, fast kernel)
    and the host-driven mixed Lanczos (generic kernel) reach the same E0, and
    both match FP64 to 1e-10 relative; fixed-step runs report every step."""
    b, s, o = make_model(qk, *m)
    H = qk.MatrixFreeHamiltonian(b, s, o)
    assert H.select_kernel(False)
    r_dev = qk.lanczos_ground_state(H, maxiter=300, tol=1e-12, mixed=True)
    r64 = qk.lanczos_ground_state(H, maxiter=300, tol=1e-12)
    H.select_kernel(True)
    r_host = qk.lanczos_ground_state(H, maxiter=300, tol=1e-12, mixed=True)
    for r in (r_dev, r_host):
        assert abs(r.energy - r64.energy) <= 1e-10 * abs(r64.energy)
        assert r.residual < 1e-4
    H.select_kernel(False)
    f = qk.lanczos_fixed_steps(H, 60, seed=3, mixed=True)
    assert f.iterations == 60 and f.spmv_calls >= 1
    assert abs(f.energy - r64.energy) <= 1e-10 * abs(r64.energy)


def test_krylov_workspace_reused_across_runs(qk):
    """The mixed Lanczos keeps its Krylov space on the Hamiltonian: a second
    run with the same seed reuses it (no fresh allocation) and reproduces the
    first bit for bit (nothing depends on the stale contents); a shorter run
    fits in it; release frees it."""
    b, s, o = make_model(qk, *M.heisenberg(18, True, 0))
    H = qk.MatrixFreeHamiltonian(b, s, o)
    assert H.workspace_bytes() == 0
    f1 = qk.lanczos_fixed_steps(H, 40, seed=5, mixed=True)
    nbytes = H.workspace_bytes()
    stride = (H.dimension + 31) // 32 * 32
    # 41 Krylov vectors, 4 Ritz-vector slots, the FP32 Ritz vector, two FP64 vectors
    assert nbytes == (40 + 1 + 4 + 1 + 4) * stride * 8
    f2 = qk.lanczos_fixed_steps(H, 40, seed=5, mixed=True)
    assert H.workspace_bytes() == nbytes
    assert (f1.energy, f1.energy_tridiag, f1.residual) == (f2.energy, f2.energy_tridiag, f2.residual)
    f3 = qk.lanczos_fixed_steps(H, 20, seed=5, mixed=True)
    assert H.workspace_bytes() == nbytes and f3.iterations == 20
    assert f3.energy_tridiag > f1.energy_tridiag - 1e-12  # fewer steps: a Ritz value no lower
    assert H.workspace_bytes(release=True) == 0


def test_lanczos_from_given_start_matches_oracle(qk, oracle):
    """Same start vector on both sides: E0 and iteration count of the
    reference algorithm (oracle restatement) are reproduced."""
    m = M.hubbard(6, True, 3, 3)
    b, s, o = make_model(qk, *m)
    H = qk.MatrixFreeHamiltonian(b, s, o)
    oh = OHam(oracle, *m)
    rng = np.random.default_rng(11)
    v0 = rng.normal(size=oh.dim) + 1j * rng.normal(size=oh.dim)
    r = qk.lanczos_ground_state(H, maxiter=300, tol=1e-12, v0=v0)
    import ctypes as c
    e, it, cv = c.c_double(), c.c_int(), c.c_int()
    evec = np.zeros(oh.dim, dtype=complex)
    oracle.lib.qko_lanczos_from(c.c_void_p(oh.h), v0.ctypes.data_as(c.POINTER(c.c_double)), 300, c.c_double(1e-12),
                                c.byref(e), c.byref(it), c.byref(cv), evec.ctypes.data_as(c.POINTER(c.c_double)),
                                None, None)
    assert abs(r.energy - e.value) <= E0_RTOL * abs(e.value)
    assert abs(abs(np.vdot(r.eigenvector, evec)) - 1) < 1e-8


@pytest.mark.parametrize("model,k", [("heis", 2), ("hub", 2), ("heis", 4)])
def test_davidson_mixed_vs_fp64(qk, model, k):
    # mixed form: FP32 vectors and SpMV, FP64-accurate projections, FP64-refined
    # Ritz pairs; its eigenvalues agree with the FP64 form's to well below the
    # FP32 residual (error ~ residual^2 / gap)
    if model == "heis":
        b, s, o = make_model(qk, M.SPIN, 14, M.sector(sz2=0), M.heisenberg_terms(14, True, Jz=0.9))
    else:
        b, s, o = make_model(qk, M.HUBBARD, 6, M.sector(nup=3, ndn=2), M.hubbard_terms(6, False, U=3.0))
    H = qk.MatrixFreeHamiltonian(b, s, o)
    # (k = 4: the mixed form projects four corrections per pass off the basis)
    r64 = qk.davidson_lowest_ex(H, n_eig=k, max_subspace=24, tol=1e-8, mixed=False)
    assert r64.converged and np.all(r64.residuals <= 1e-8)
    r32 = qk.davidson_lowest_ex(H, n_eig=k, max_subspace=24, tol=1e-5, mixed=True, return_vectors=True)
    assert r32.converged, r32.residuals
    assert np.all(r32.residuals <= 1e-5)
    np.testing.assert_allclose(r32.eigenvalues, r64.eigenvalues, rtol=0, atol=1e-8)
    for lam, v, res in zip(r32.eigenvalues, r32.eigenvectors, r32.residuals):
        assert abs(np.linalg.norm(v) - 1) < 1e-12
        np.testing.assert_allclose(np.linalg.norm(H.apply(v) - lam * v), res, rtol=1e-6, atol=1e-12)


@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
def test_davidson_hubbard_L10_against_lanczos(qk, mixed):
    """Davidson on the Fermi-Hubbard chain L=10 periodic, U=4, half filling
    (dim 63,504), lowest 4 states, subspace 32, block 4, tol 1e-8, the
    reference's cap of 100 iterations (src/solvers/davidson.cpp:141,180): the
    lowest eigenvalue agrees with the FP64 Lanczos E0 of the same sector within
    the Davidson residual norm (for a Hermitian operator some eigenvalue lies
    within ||r|| of a Ritz value; the lowest Ritz value is bounded below by E0)."""
    b, s, o = make_model(qk, M.HUBBARD, 10, M.sector(nup=5, ndn=5), M.hubbard_terms(10, True))
    H = qk.MatrixFreeHamiltonian(b, s, o)
    lz = qk.lanczos_ground_state(H, maxiter=300, tol=1e-13)
    assert lz.converged
    r = qk.davidson_lowest_ex(H, n_eig=4, max_subspace=32, tol=1e-8, mixed=mixed, max_iter=100)
    assert r.iterations <= 100
    lam0, res0 = float(r.eigenvalues[0]), float(r.residuals[0])
    assert lam0 >= lz.energy - 1e-10 * abs(lz.energy)  # Rayleigh-Ritz: no Ritz value below E0
    assert lam0 - lz.energy <= res0 + 1e-10 * abs(lz.energy), (lam0, lz.energy, res0)
    assert np.all(np.diff(r.eigenvalues) >= -1e-12)


def _random_chain(qk, L, seed):
    """Open Heisenberg chain with random bonds and random longitudinal fields
    (Sz conserved, no spatial symmetry: no degenerate levels)."""
    rng = np.random.default_rng(seed)
    ops = qk.OpSum()
    for i in range(L - 1):
        J = 0.5 + rng.random()
        ops.add_term(J, "Sz", i, "Sz", i + 1)
        ops.add_term(0.5 * J, "Sp", i, "Sm", i + 1)
        ops.add_term(0.5 * J, "Sm", i, "Sp", i + 1)
    for i in range(L):
        ops.add_term(0.3 * (rng.random() - 0.5), "Sz", i)
    return qk.MatrixFreeHamiltonian(qk.SpinHalfBasis(L, conserve_sz=True, sz=0), qk.SpinHalfSite(), ops)


def test_selective_reorth_holds_several_ritz_vectors(qk):
    # Parlett-Scott selective reorthogonalisation against every converged low
    # Ritz vector (up to four): after many more steps than the ground state
    # needs, the lowest Ritz values of the mixed form (FP32) and of FP64 with
    # selective reorthogonalisation are those of FP64 with full
    # reorthogonalisation and of the dense spectrum -- no ghost copies of a
    # converged level among them
    H = _random_chain(qk, 14, seed=11)  # dim 3432
    exact = np.linalg.eigvalsh(H.to_sparse().toarray())[:5]
    full, n0 = qk.lanczos_ritz_values(H, 300, 5, seed=3, mixed=False)
    sel, n64 = qk.lanczos_ritz_values(H, 300, 5, seed=3, mixed=False, selective=True)
    mix, n32 = qk.lanczos_ritz_values(H, 300, 5, seed=3, mixed=True)
    assert n0 == 0
    assert n64 >= 2 and n32 >= 2, (n64, n32)  # more than the ground state's Ritz vector is held
    np.testing.assert_allclose(full, exact, rtol=0, atol=1e-9)
    np.testing.assert_allclose(sel, exact, rtol=0, atol=1e-9)
    np.testing.assert_allclose(mix, exact, rtol=0, atol=5e-5)  # FP32 vectors
