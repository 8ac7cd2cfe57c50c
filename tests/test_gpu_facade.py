"""The Python facade's matrix conversions, with the reference facade's
semantics (bindings/python/qkrylov/hamiltonian.py:120-177): to_sparse() is
the matrix whose column i is H e_i (the reference builds it that way, one
apply per unit vector), aslinearoperator() a SciPy LinearOperator whose matvec
is H.apply."""
import numpy as np
import pytest

import models as M
from conftest import golden_terms, load_golden, make_model

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["heis_L10_pbc_sz0", "hub_L4_full", "ferm_L8_full", "xyz_L8_sz0", "tj_L5_full"])
def test_to_sparse_equals_columns_of_apply(qk, name):
    sp = pytest.importorskip("scipy.sparse")
    g = load_golden(name)
    b, s, o = make_model(qk, g["model"], g["nsites"], g["sector"], golden_terms(g))
    H = qk.MatrixFreeHamiltonian(b, s, o)
    n = H.dimension
    A = H.to_sparse()
    assert sp.issparse(A) and A.shape == (n, n)
    dense = A.toarray()
    # the reference facade's construction: column i = H e_i
    cols = np.zeros((n, n), dtype=complex)
    for i in range(n):
        e = np.zeros(n, dtype=complex)
        e[i] = 1.0
        cols[:, i] = H.apply(e)
    np.testing.assert_allclose(dense, cols, rtol=0, atol=1e-14)  # equal up to the order of the diagonal sums
    # and the reference's own CSR (golden, duplicates summed)
    ref = sp.csr_matrix((g["csr_vals"], g["csr_cols"].astype(np.int64), g["csr_ro"].astype(np.int64)), shape=(n, n))
    np.testing.assert_allclose(dense, ref.toarray(), rtol=0, atol=1e-14)


def test_aslinearoperator_matvec_and_eigsh(qk):
    sla = pytest.importorskip("scipy.sparse.linalg")
    b, s, o = make_model(qk, *M.heisenberg(14, True, 0))
    H = qk.MatrixFreeHamiltonian(b, s, o)
    op = H.aslinearoperator()
    n = H.dimension
    assert op.shape == (n, n) and op.dtype == np.complex128
    rng = np.random.default_rng(4)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    assert np.array_equal(op @ x, H.apply(x))
    e0 = qk.lanczos_ground_state(H, maxiter=300, tol=1e-13).energy
    w = sla.eigsh(op, k=1, which="SA", tol=1e-12, return_eigenvectors=False)
    assert abs(float(w[0]) - e0) <= 1e-9 * abs(e0)
