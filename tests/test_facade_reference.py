"""The Python facade against the reference facade's own tests
(bindings/python/tests/test_basic.py, test_workflow.py and
tests/python/test_scipy.py), restated for this package: the same calls, the
same expected answers.  Bases and the operator algebra run on the host; the
Hamiltonian cases need the GPU."""
import math

import numpy as np
import pytest


def test_bases_as_the_reference_facade(qk):
    # test_basic.py:4-31
    basis = qk.SpinHalfBasis(4)
    assert basis.size == 16 and basis.nsites == 4
    assert qk.FermionBasis(4, conserve_n=True, n=2).size == 6
    assert qk.TJBasis(2).size == 9
    # the facade's sector rules (basis.py:64-190): an explicit quantum number
    # conserves it, n = 0 alone does not, species are independent
    assert qk.SpinHalfBasis(N=4, sz=0).size == 6
    assert qk.SpinHalfBasis(4, conserve_sz=True).size == 6
    assert qk.FermionBasis(4, n=0).size == 16
    assert qk.FermionBasis(4, conserve_n=True).size == 1
    assert qk.HubbardBasis(4, nup=2).size == 6 * 16
    assert qk.HubbardBasis(4, nup=2, ndn=1).size == 6 * 4
    assert qk.HubbardBasis(4, conserve_nup=True, nup=2, conserve_ndn=True, ndn=2, dtype=np.float64).size == 36
    assert qk.TJBasis(3, nup=1, ndn=1).size == 6
    qk.SpinHalfSite(dtype=np.float64)


def test_operator_algebra_as_the_reference_facade(qk):
    # test_workflow.py:14-21: three bonds of 1.0 Sz Sz + 0.5 (Sp Sm + Sm Sp)
    ops = qk.OpSum()
    for i in range(3):
        ops += 1.0 * qk.Sz(i) * qk.Sz(i + 1) + 0.5 * (qk.Sp(i) * qk.Sm(i + 1) + qk.Sm(i) * qk.Sp(i + 1))
    assert ops.size == 9
    assert ops.terms[1] == (0.5, [("Sp", 0), ("Sm", 1)])
    # subtraction and scaling of sums (operators.py:64-110), Op names
    e = qk.Sz(0) * qk.Sz(1) - 2.0 * (1.0 * qk.Sx(0) + qk.Sx(1) * 1.0)
    assert [t.coeff for t in e.terms] == [1.0, -2.0, -2.0]
    ops2 = qk.OpSum()
    ops2.add_term(0.25, qk.Op.Sz, 0, qk.Op.Sz, 1)
    assert ops2.terms == [(0.25, [("Sz", 0), ("Sz", 1)])]
    # an operator on the left of a product stays on the left
    t = qk.Sz(0) * (qk.Sp(1) * qk.Sm(2))
    assert [(o.name, o.site) for o in t.ops] == [("Sz", 0), ("Sp", 1), ("Sm", 2)]
    # test_basic.py:33-41: malformed += raises ValueError
    ops3 = qk.OpSum()
    ops3 += (1.0, "Sz", 0, "Sz", 1)
    with pytest.raises(ValueError):
        ops3 += (1.0, "Sz")
    with pytest.raises(ValueError):
        ops3 += 3
    ops3.clear()
    assert ops3.size == 0


def test_device_helpers(qk):
    assert qk.Device("cuda:1").id == 1 and qk.Device(2).id == 2 and qk.Device("cpu").id == 0
    assert qk.Device.is_gpu_build() and qk.Device.backend_name() == "cuda"
    n = qk.gpu_count()
    assert n >= 0 and qk.find_gpu() == ("cuda" if n else None)


@pytest.mark.gpu
def test_hamiltonian_and_workflow_as_the_reference_facade(qk):
    # test_basic.py:14-24
    basis = qk.SpinHalfBasis(2)
    ops = qk.OpSum()
    ops.add_term(1.0, "Sz", 0, "Sz", 1)
    H = qk.MatrixFreeHamiltonian(basis, qk.SpinHalfSite(), ops)
    assert H.dimension == 4 and len(H.diagonal()) == 4
    # test_basic.py:43-47: a vector of the wrong length raises ValueError
    with pytest.raises(ValueError):
        H.apply(np.zeros(10, dtype=np.complex128))
    # test_workflow.py:5-31: 4-site open chain, Sz = 0, E0 = -1.6160254038
    basis = qk.SpinHalfBasis(N=4, sz=0)
    ops = qk.OpSum()
    for i in range(3):
        ops += 1.0 * qk.Sz(i) * qk.Sz(i + 1) + 0.5 * (qk.Sp(i) * qk.Sm(i + 1) + qk.Sm(i) * qk.Sp(i + 1))
    H = qk.MatrixFreeHamiltonian(basis, qk.SpinHalfSite(), ops)
    assert H.dimension == 6
    res = qk.lanczos_ground_state(H, 200, 1e-12)
    assert math.isclose(res.energy, -1.6160254038, abs_tol=1e-5)
    assert len(res.eigenvector) == 6


@pytest.mark.gpu
def test_scipy_conversions_and_to_as_the_reference_facade(qk):
    # tests/python/test_scipy.py:4-27
    pytest.importorskip("scipy.sparse.linalg")
    basis = qk.SpinHalfBasis(2, sz=0)
    ops = qk.OpSum()
    ops += 1.0 * qk.Sz(0) * qk.Sz(1) + 0.5 * (qk.Sp(0) * qk.Sm(1) + qk.Sm(0) * qk.Sp(1))
    H = qk.MatrixFreeHamiltonian(basis, qk.SpinHalfSite(), ops)
    assert H.dimension > 0
    assert H.aslinearoperator().shape == (H.dimension, H.dimension)
    assert H.to_sparse().shape == (H.dimension, H.dimension)
    H2 = H.to(device="cpu")
    assert H2.dimension == H.dimension
    x = np.random.default_rng(0).random(H.dimension)
    np.testing.assert_allclose(H.apply(x), H2 @ x)
    # dtype=np.float32: complex64 results, the same values rounded
    H32 = H.to(dtype=np.float32)
    y32 = H32 @ x
    assert y32.dtype == np.complex64
    np.testing.assert_allclose(y32, H.apply(x), rtol=1e-6, atol=1e-7)
    with pytest.raises(ValueError):
        H.to(device="tpu")
