"""Eigenvector / tridiagonal files: the formats on the host, and a GPU ground
state and continued fraction written, read back and reused."""
import numpy as np
import pytest

import models as M


def test_eigenvector_roundtrip_and_basis_check(qk, tmp_path):
    b = qk.SpinHalfBasis(12, conserve_sz=True, sz=0)
    other = qk.SpinHalfBasis(12, conserve_sz=True, sz=1)
    rng = np.random.default_rng(0)
    v = rng.normal(size=(2, b.size)) + 1j * rng.normal(size=(2, b.size))
    p = str(tmp_path / "ev.npz")
    qk.io.save_eigenvector(p, v, [-5.0, -4.5], b, extra={"seed": 3})
    vv, ee, meta = qk.io.load_eigenvector(p, b)
    np.testing.assert_array_equal(vv, v)
    np.testing.assert_array_equal(ee, [-5.0, -4.5])
    assert meta["sector"] == {"sz2": 0} and meta["extra"] == {"seed": 3} and meta["dim"] == b.size
    with pytest.raises(ValueError):
        qk.io.load_eigenvector(p, other)
    with pytest.raises(ValueError):
        qk.io.save_eigenvector(p, v[:, :-1], [0.0, 0.0], b)


def test_hubbard_signature_uses_reference_states(qk, tmp_path):
    b = qk.HubbardBasis(5, nup=2, ndn=2)
    sig = qk.io.basis_signature(b)
    assert sig["dim"] == 100 and sig["model"] == "HubbardBasis"
    st = b.states()
    assert np.all(np.diff(st.astype(np.int64)) > 0)  # ascending interleaved reference order
    assert st[0] == b.state(0) and st[-1] == b.state(b.size - 1)


def test_tridiagonals_roundtrip(qk, tmp_path):
    res = [(np.array([1.0, 2.0, 3.0]), np.array([0.5, 0.25]), 2.0), (np.zeros(0), np.zeros(0), 0.0)]
    b = qk.SpinHalfBasis(6, conserve_sz=True, sz=0)
    p = str(tmp_path / "cf.npz")
    qk.io.save_tridiagonals(p, res, b)
    back, meta = qk.io.load_tridiagonals(p, b)
    assert len(back) == 2 and meta["kind"] == "tridiagonals"
    for (a0, b0, n0), (a1, b1, n1) in zip(res, back):
        np.testing.assert_array_equal(a0, a1)
        np.testing.assert_array_equal(b0, b1)
        assert n0 == n1
    with pytest.raises(ValueError):
        qk.io.load_eigenvector(p)


@pytest.mark.gpu
def test_ground_state_checkpoint_and_restart(qk, tmp_path):
    # a GPU ground state written to a file and read back is still an
    # eigenvector of H, and a Lanczos run restarted from it converges at once
    basis, site, ops = M.make_model(qk, *M.heisenberg(16, True, 0))
    H = qk.MatrixFreeHamiltonian(basis, site, ops)
    r = qk.lanczos_ground_state(H, maxiter=300, tol=1e-13)
    p = str(tmp_path / "gs.npz")
    qk.io.save_eigenvector(p, r.eigenvector[None, :], [r.energy], basis, extra={"iterations": r.iterations})
    v, e, meta = qk.io.load_eigenvector(p, basis)
    psi = v[0]
    hpsi = H.apply(psi)
    assert np.linalg.norm(hpsi - e[0] * psi) < 1e-5
    assert abs(np.vdot(psi, hpsi).real - r.energy) < 1e-10 * abs(r.energy)
    again = qk.lanczos_ground_state(H, maxiter=300, tol=1e-13, v0=psi)
    assert abs(again.energy - r.energy) < 1e-10 * abs(r.energy)
    assert again.iterations < r.iterations


@pytest.mark.gpu
def test_continued_fraction_file_gives_the_same_spectrum(qk, tmp_path):
    # S(omega) evaluated from tridiagonals written and read back equals the
    # value from the GPU run itself
    basis, site, ops = M.make_model(qk, *M.heisenberg(12, True, 0))
    H = qk.MatrixFreeHamiltonian(basis, site, ops)
    gs = qk.lanczos_ground_state(H, maxiter=200, tol=1e-12)
    phi = gs.eigenvector * np.linspace(0.5, 1.5, H.dimension)
    cf = qk.continued_fraction_coeffs(H, phi, n_iter=80)
    p = str(tmp_path / "cf.npz")
    qk.io.save_tridiagonals(p, [(cf.alphas, cf.betas, cf.norm_phi0)], basis)
    (a, bb, nrm), = qk.io.load_tridiagonals(p, basis)[0]
    back = qk.DynamicsResult(a, bb, nrm)
    om = np.linspace(0.0, 4.0, 41)
    np.testing.assert_array_equal(qk.evaluate_spectral_function(back, om, gs.energy, 0.1),
                                  qk.evaluate_spectral_function(cf, om, gs.energy, 0.1))
