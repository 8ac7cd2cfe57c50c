"""Eigenvector / tridiagonal files (CPU: bases are host objects)."""
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
