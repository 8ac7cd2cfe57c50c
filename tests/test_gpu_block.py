"""Batched (block-vector) Lanczos: FTLM over all Sz sectors in one run and
continued fractions for several right-hand sides, against the oracle's
single-vector restatement of ftlm.cpp / dynamics.cpp."""
import numpy as np
import pytest

import models as M
from conftest import make_model
from oracle_ctypes import OHam, spectral

pytestmark = pytest.mark.gpu

EARLY_RTOL = 1e-10   # FP64 alphas/betas of the first steps (before loss of orthogonality amplifies rounding)
OBS_RTOL = 1e-8      # FP64 Z, E, Cv and S(omega)
# FP32 Krylov vectors with FP64-accurate reductions against the FP64 form: the
# bounds are about five times the largest errors measured on GB300 at these
# sizes and at L = 10..18 (FTLM: relative dZ <= 6.1e-7, |dE| <= 7.3e-8,
# |dCv| <= 2.0e-7; S(omega): relative <= 3.6e-6).  They sit at the FP32
# storage rounding of the vectors (2^-24 = 6e-8) times each observable's
# conditioning, which no reduction accuracy removes; the FP64 forms are held
# to OBS_RTOL.
MIXED_Z_RTOL = 3e-6
MIXED_E_ATOL = 4e-7
MIXED_CV_ATOL = 1e-6
MIXED_S_RTOL = 2e-5


def chain_sectors(qk, L, pbc=True):
    hams, models = [], []
    for sz2 in range(-L, L + 1, 2):
        sec = M.sector(sz2=sz2)
        terms = M.heisenberg_terms(L, pbc)
        b, s, o = make_model(qk, M.SPIN, L, sec, terms)
        hams.append(qk.MatrixFreeHamiltonian(b, s, o))
        models.append((M.SPIN, L, sec, terms))
    return hams, models


def combine(parts, betas):
    """Sum of per-sector FTLM estimates (Z_s, E_s, Cv_s) into the ensemble's."""
    Z = sum(p[0] for p in parts)
    E = sum(p[0] * p[1] for p in parts) / Z
    E2 = sum(p[0] * (p[2] / betas ** 2 + p[1] ** 2) for p in parts) / Z
    return Z, E, betas ** 2 * (E2 - E ** 2)


def test_block_fp64_tridiagonals_match_oracle(qk, oracle):
    L, R, Mst = 10, 3, 15
    hams, models = chain_sectors(qk, L)
    res = qk.block_lanczos_tridiag(hams, R, Mst, mixed=False, start="ftlm")
    assert res.stats["padded_vectors"] == 4
    for h, m in enumerate(models):
        a, b, na, nb, nr = OHam(oracle, *m).ftlm_tridiag(R, Mst)
        for v in range(R):
            i = h * R + v
            np.testing.assert_allclose(res.norm2[i], nr[v] ** 2, rtol=1e-12)
            ga, gb = res.alphas[i], res.betas[i]
            scale = max(1.0, np.abs(a[v, :na[v]]).max())
            # steps before the Krylov space closes (beta at rounding level, where
            # the 1e-15 stop decides on noise): they must agree
            ob = b[v, :nb[v]]
            closed = np.nonzero(ob < 1e-8 * scale)[0]
            kb = min(8, len(gb), int(closed[0]) if closed.size else nb[v])
            k = min(kb + 1, na[v], len(ga))
            assert k >= 1
            assert np.abs(ga[:k] - a[v, :k]).max() <= EARLY_RTOL * scale
            if kb:
                assert np.abs(gb[:kb] - ob[:kb]).max() <= EARLY_RTOL * scale
            if not closed.size and hams[h].dimension > Mst:
                assert len(ga) == na[v] and len(gb) == nb[v]


def test_block_sector_batch_equals_single(qk):
    hams, _ = chain_sectors(qk, 12)
    both = qk.block_lanczos_tridiag([hams[5], hams[6]], 4, 20, mixed=True, start="philox", seed=9)
    one = qk.block_lanczos_tridiag([hams[5]], 4, 20, mixed=True, start="philox", seed=9)
    for v in range(4):
        np.testing.assert_array_equal(both.alphas[v], one.alphas[v])
        np.testing.assert_array_equal(both.betas[v], one.betas[v])


def test_block_philox_deterministic(qk):
    hams, _ = chain_sectors(qk, 12)
    r1 = qk.block_lanczos_tridiag(hams, 8, 12, mixed=True, start="philox", seed=5)
    r2 = qk.block_lanczos_tridiag(hams, 8, 12, mixed=True, start="philox", seed=5)
    r3 = qk.block_lanczos_tridiag(hams, 8, 12, mixed=True, start="philox", seed=6)
    for i in range(len(r1.alphas)):
        np.testing.assert_array_equal(r1.alphas[i], r2.alphas[i])
    mid = len(hams) // 2 * 8
    assert not np.array_equal(r1.alphas[mid], r3.alphas[mid])
    # Gaussian complex start vectors: E|x|^2 = 2 per component
    dims = np.repeat([h.dimension for h in hams], 8)
    big = dims >= 500
    assert np.all(np.abs(r1.norm2[big] / (2 * dims[big]) - 1) < 0.2)


def test_ftlm_sectors_fp64_matches_oracle(qk, oracle):
    L, R, Mst = 10, 4, 20
    betas = np.array([0.1, 0.5, 1.0, 3.0])
    hams, models = chain_sectors(qk, L)
    r = qk.ftlm_sectors(hams, betas, n_random=R, n_steps=Mst, mixed=False, start="ftlm")
    parts = []
    for m in models:
        o = OHam(oracle, *m)
        z = np.array([o.ftlm(b, R, Mst) for b in betas])
        parts.append((z[:, 0], z[:, 1], z[:, 2]))
    Z, E, C = combine(parts, betas)
    np.testing.assert_allclose(r.partition_function, Z, rtol=OBS_RTOL)
    np.testing.assert_allclose(r.internal_energy, E, rtol=OBS_RTOL, atol=OBS_RTOL)
    np.testing.assert_allclose(r.specific_heat, C, rtol=OBS_RTOL, atol=OBS_RTOL)
    s = qk.ftlm_sectors(hams, betas, n_random=R, n_steps=Mst, mixed=False, start="ftlm", shifted=True)
    np.testing.assert_allclose(s.partition_function * np.exp(s.log_shift), Z, rtol=OBS_RTOL)
    np.testing.assert_allclose(s.specific_heat, C, rtol=OBS_RTOL, atol=OBS_RTOL)


def test_ftlm_sectors_mixed_vs_fp64(qk):
    L, R, Mst = 14, 8, 40
    betas = np.geomspace(0.1, 10.0, 7)
    hams, _ = chain_sectors(qk, L)
    r64 = qk.ftlm_sectors(hams, betas, n_random=R, n_steps=Mst, mixed=False, start="ftlm", shifted=True)
    r32 = qk.ftlm_sectors(hams, betas, n_random=R, n_steps=Mst, mixed=True, start="ftlm", shifted=True)
    z64 = r64.partition_function * np.exp(r64.log_shift - r64.log_shift)
    z32 = r32.partition_function * np.exp(r32.log_shift - r64.log_shift)
    np.testing.assert_allclose(z32, z64, rtol=MIXED_Z_RTOL)
    np.testing.assert_allclose(r32.internal_energy, r64.internal_energy, rtol=0, atol=MIXED_E_ATOL)
    np.testing.assert_allclose(r32.specific_heat, r64.specific_heat, rtol=0, atol=MIXED_CV_ATOL)


@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
def test_cf_block_matches_oracle(qk, oracle, mixed):
    # Hubbard chain: a permuted basis, so the start vectors go through the
    # reference-to-internal permutation
    L, n_iter = 6, 30
    m = (M.HUBBARD, L, M.sector(nup=3, ndn=3), M.hubbard_terms(L, True))
    b, s, o = make_model(qk, *m)
    H = qk.MatrixFreeHamiltonian(b, s, o)
    n = H.dimension
    rng = np.random.default_rng(3)
    phis = rng.normal(size=(5, n)) + 1j * rng.normal(size=(5, n))
    phis[2] = 0.0  # a zero right-hand side gets no coefficients (dynamics.cpp:27)
    res, stats = qk.continued_fraction_block(H, phis, n_iter=n_iter, mixed=mixed)
    assert stats["padded_vectors"] == 8
    oh = OHam(oracle, *m)
    omegas = np.linspace(-2.0, 8.0, 41)
    for i in range(5):
        a, bb, nrm = oh.cf(phis[i], n_iter)
        if i == 2:
            assert res[i].norm_phi0 == 0.0 and len(res[i].alphas) == 0
            continue
        np.testing.assert_allclose(res[i].norm_phi0, nrm, rtol=1e-12 if not mixed else 1e-6)
        assert len(res[i].alphas) == len(a) and len(res[i].betas) == len(bb)
        if not mixed:
            k = min(10, len(a))
            assert np.abs(res[i].alphas[:k] - a[:k]).max() <= EARLY_RTOL * max(1.0, np.abs(a).max())
        S = np.array([qk.evaluate_spectral_function(res[i], w, -3.0, eta=0.2) for w in omegas])
        So = np.array([spectral(oracle, a, bb, nrm, w, -3.0, 0.2) for w in omegas])
        tol = OBS_RTOL if not mixed else MIXED_S_RTOL
        assert np.abs(S - So).max() <= tol * np.abs(So).max()


def test_block_rejects_bad_arguments(qk):
    hams, _ = chain_sectors(qk, 6)
    with pytest.raises(qk.QKrylovError):
        qk.block_lanczos_tridiag(hams, 33, 4)
    with pytest.raises(qk.QKrylovError):
        qk.ftlm_sectors(hams, [1.0], n_random=0)


@pytest.mark.parametrize("R", [1, 2, 8, 32])
def test_block_tile_shapes_agree(qk, R):
    # every vectors-per-lane tile computes the same row sums; only the order of
    # the per-CTA reduction partials differs
    hams, _ = chain_sectors(qk, 12)
    ref = None
    for vpl in (1, 2, 4):
        if R % vpl or R // vpl > 32:
            continue
        r = qk.block_lanczos_tridiag(hams, R, 10, mixed=False, start="philox", seed=2, vpl=vpl)
        assert r.stats["vectors_per_lane"] == vpl
        if ref is None:
            ref = r
            continue
        for i in range(len(r.alphas)):
            n = min(len(r.alphas[i]), len(ref.alphas[i]), 6)
            assert np.abs(r.alphas[i][:n] - ref.alphas[i][:n]).max(initial=0) <= 1e-12 * 8


@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
def test_structure_factor_block(qk, oracle, mixed):
    # S(q, omega) right-hand sides Sz(q)|psi0> built by applying an OpSum
    # operator to the ground state; all q in one batched run
    L = 10
    m = (M.SPIN, L, M.sector(sz2=0), M.heisenberg_terms(L, True))
    b, s, o = make_model(qk, *m)
    H = qk.MatrixFreeHamiltonian(b, s, o)
    gs = qk.lanczos_ground_state(H, maxiter=200, tol=1e-12)
    psi, E0 = gs.eigenvector, gs.energy
    st = b.states()
    assert st.size == H.dimension and np.array_equal(st[:3], [b.state(i) for i in range(3)])
    sz = ((st[:, None] >> np.arange(L, dtype=np.uint64)) & np.uint64(1)).astype(float) - 0.5
    phis = []
    for k in range(L // 2 + 1):
        ph = np.exp(2j * np.pi * k / L * np.arange(L)) / np.sqrt(L)
        ops = qk.OpSum()
        for j in range(L):
            ops.add_term(ph[j], "Sz", j)
        phi = qk.MatrixFreeHamiltonian(b, qk.SpinHalfSite(), ops).apply(psi)
        # the matrix elements are the conjugated term amplitudes
        # (matrix_free_hamiltonian.cpp stores conj(amp)), so this applies Sz(-q)
        np.testing.assert_allclose(phi, psi * (sz @ np.conj(ph)), atol=1e-13)
        phis.append(phi)
    omegas = np.linspace(0.0, 4.0, 81)
    S, res, stats = qk.spectral_functions_block(H, phis, omegas, E0, eta=0.05, n_iter=60, mixed=mixed)
    assert np.all(S[0] == 0.0) and res[0].norm_phi0 == 0.0  # q = 0: total Sz = 0 in this sector
    oh = OHam(oracle, *m)
    for k in range(1, len(phis)):
        a, bb, nrm = oh.cf(phis[k], 60)
        So = np.array([spectral(oracle, a, bb, nrm, w, E0, 0.05) for w in omegas])
        tol = OBS_RTOL if not mixed else MIXED_S_RTOL
        assert np.abs(S[k] - So).max() <= tol * np.abs(So).max()


def test_ftlm_sectors_host_reduction_matches(qk):
    # the sharded path's host reduction (one rank here) against the library's
    from qkrylov_gb300.parallel import ftlm_sectors_distributed
    L, R, Mst = 10, 4, 20
    betas = np.array([0.1, 1.0, 4.0])
    hams, _ = chain_sectors(qk, L)
    sizes = [h.dimension for h in hams]
    Z, E, C, ls = ftlm_sectors_distributed(lambda idx: [hams[i] for i in idx], sizes, betas, n_random=R,
                                           n_steps=Mst, mixed=False, start="ftlm")
    r = qk.ftlm_sectors(hams, betas, n_random=R, n_steps=Mst, mixed=False, start="ftlm", shifted=True)
    np.testing.assert_allclose(Z * np.exp(ls), r.partition_function * np.exp(r.log_shift), rtol=1e-9)
    np.testing.assert_allclose(E, r.internal_energy, rtol=1e-9, atol=1e-9)
    np.testing.assert_allclose(C, r.specific_heat, rtol=1e-8, atol=1e-8)
