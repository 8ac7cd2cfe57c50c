"""The oracle restatement is pinned to the reference: against the golden
fixtures the reference produced (tests/golden/, make_golden.py), against the
known answers in the reference's own tests, and, where the reference build
exists in this checkout (oracle/_ref), against the reference directly."""
import numpy as np
import pytest

import models as M
from conftest import golden_names, golden_terms, load_golden
from oracle_ctypes import OHam, Oracle, available, spectral

NAMES = golden_names()


def _ham(oracle, g):
    return OHam(oracle, int(g["model"]), int(g["nsites"]), [int(v) for v in g["sector"]], golden_terms(g))


@pytest.mark.parametrize("name", NAMES)
def test_basis_and_entries_bit_exact(oracle, name):
    g = load_golden(name)
    h = _ham(oracle, g)
    assert h.dim == int(g["dim"])
    assert np.array_equal(h.states(), g["states"])
    if "csr_ro" in g:
        ro, cols, vals = h.csr()
        assert np.array_equal(ro, g["csr_ro"])
        assert np.array_equal(cols, g["csr_cols"])
        assert np.array_equal(vals, g["csr_vals"])
        y = h.apply(g["x"])
        assert np.array_equal(y, g["y"])
    assert np.array_equal(h.diagonal(), g["diag"])


@pytest.mark.parametrize("name", NAMES)
def test_solvers_match_reference(oracle, name):
    g = load_golden(name)
    h = _ham(oracle, g)
    e, it, cv, v = h.lanczos(300, 1e-12)
    assert abs(e - g["lanczos_E0"]) <= 1e-10 * max(1.0, abs(g["lanczos_E0"]))
    ev, *_ = h.davidson(len(g["davidson_evals"]), 20, 1e-8)
    np.testing.assert_allclose(ev, g["davidson_evals"], rtol=1e-8, atol=1e-8)
    if "cf_phi0" in g:
        a, b, nrm = h.cf(g["cf_phi0"], len(g["cf_alphas"]))
        k = min(10, len(a))
        np.testing.assert_allclose(a[:k], g["cf_alphas"][:k], rtol=1e-9, atol=1e-9)
        np.testing.assert_allclose(b[:k], g["cf_betas"][:k], rtol=1e-9, atol=1e-9)
        assert abs(nrm - g["cf_norm"]) <= 1e-12 * g["cf_norm"]
    R, Mst = g["ftlm_alphas"].shape
    ta, tb, na, nb, nr = h.ftlm_tridiag(R, Mst)
    np.testing.assert_allclose(nr, g["ftlm_norms"], rtol=1e-13)
    np.testing.assert_array_equal(na, g["ftlm_na"])
    for r in range(R):
        k = min(8, int(na[r]))
        np.testing.assert_allclose(ta[r, :k], g["ftlm_alphas"][r, :k], rtol=1e-9, atol=1e-9)
    for bt, obs in zip(g["ftlm_betas_T"], g["ftlm_obs"]):
        np.testing.assert_allclose(h.ftlm(bt, R, Mst), obs, rtol=1e-8)


def test_reference_known_answers(oracle):
    # tests/test_workflow.cpp:22-49: 4-site OBC chain, Sz=0, E0 = -1.6160254038
    h = OHam(oracle, *M.heisenberg(4, False, 0))
    assert h.dim == 6
    assert abs(h.lanczos(200, 1e-12)[0] + 1.6160254038) < 1e-5
    # tests/test_lanczos_ritz.cpp:43-55: 2-site full basis, E0 = -0.75
    h = OHam(oracle, *M.heisenberg(2, False, None))
    assert abs(h.lanczos(200, 1e-12)[0] + 0.75) < 1e-5
    # tests/test_fermion_basis.cpp:10-20 and test_tj_basis.cpp:12-14 dims
    assert OHam(oracle, M.FERMION, 4, M.sector(), [(1.0, [("N", 0)])]).dim == 16
    assert OHam(oracle, M.FERMION, 4, M.sector(n=2), [(1.0, [("N", 0)])]).dim == 6
    assert OHam(oracle, M.TJ, 2, M.sector(), [(1.0, [("Nup", 0)])]).dim == 9
    # tests/test_fermion_site.cpp:19-26: C on site 3 of 0b1010 -> -1, new state 0b0010
    h = OHam(oracle, M.FERMION, 4, M.sector(), [(1.0, [("C", 3)])])
    ro, cols, vals = h.csr()
    a, b = h.index(0b1010), h.index(0b0010)
    assert list(cols[ro[a]:ro[a + 1]]) == [b] and vals[ro[a]] == -1.0
    # tests/test_tj_site.cpp:12-18: CUp on 0b0001 -> +1 to 0; CdagDn onto the occupied site is invalid
    h = OHam(oracle, M.TJ, 2, M.sector(), [(1.0, [("CUp", 0)])])
    ro, cols, vals = h.csr()
    a = h.index(0b0001)
    assert list(cols[ro[a]:ro[a + 1]]) == [h.index(0)] and vals[ro[a]] == 1.0
    h = OHam(oracle, M.TJ, 2, M.sector(), [(1.0, [("CdagDn", 0)])])
    ro, _, _ = h.csr()
    a = h.index(0b0001)
    assert ro[a + 1] == ro[a]
    # bindings/julia/test/runtests.jl:106: 3-site full basis, Sz0 Sz1 + 0.5 Sz0 Sz1 Sz2 on |111> -> 0.3125
    h = OHam(oracle, M.SPIN, 3, M.sector(), [(1.0, [("Sz", 0), ("Sz", 1)]),
                                             (0.5, [("Sz", 0), ("Sz", 1), ("Sz", 2)])])
    x = np.zeros(8, dtype=complex)
    x[7] = 1.0
    assert abs(h.apply(x)[7] - 0.3125) < 1e-12


def test_capi_golden_values():
    # The reference C API (FP32 engine) on tests/test_c_api.cpp's chain.
    g = dict(np.load(__import__("conftest").GOLDEN + "/capi_heis4.npz"))
    assert int(g["dim"]) == 6
    assert abs(float(g["energy"]) + 1.6160254038) < 1e-5
    assert abs(float(g["dav_evals"][0]) - float(g["energy"])) < 1e-4
    assert float(g["s05"]) > 0 and float(g["ftlm"][1]) > 0


def test_spectral_function_matches_formula(oracle):
    a = np.array([0.3, -0.2, 0.5])
    b = np.array([0.4, 0.25, 0.0])
    z = complex(0.7 - 1.1, 0.05)
    f = 1 / (z - a[2])
    f = 1 / (z - a[1] - b[1] ** 2 * f)
    f = 1 / (z - a[0] - b[0] ** 2 * f)
    assert abs(spectral(oracle, a, b, 1.3, 0.7, -1.1, 0.05) - (-1 / np.pi * (1.3 ** 2 * f).imag)) < 1e-14


@pytest.mark.skipif(not available("qkref64"), reason="reference build (oracle/_ref) not present")
@pytest.mark.parametrize("seed", range(6))
def test_random_models_against_reference(oracle, seed):
    ref = Oracle("qkref64")
    rng = np.random.default_rng(seed)
    model = [M.SPIN, M.FERMION, M.HUBBARD, M.TJ][seed % 4]
    ops = {M.SPIN: ["Sz", "Sp", "Sm", "Sx", "Sy"], M.FERMION: ["N", "Id", "C", "Cdag"],
           M.HUBBARD: ["Nup", "Ndn", "Nupdn", "CUp", "CdagUp", "CDn", "CdagDn"],
           M.TJ: ["Nup", "Ndn", "CUp", "CdagUp", "CDn", "CdagDn"]}[model]
    N = 7 if model < 2 else 4
    terms = []
    for _ in range(25):
        nf = int(rng.integers(1, 5))
        terms.append((complex(rng.normal(), rng.normal() * (seed % 2)),
                      [(str(rng.choice(ops)), int(rng.integers(0, N))) for _ in range(nf)]))
    sector = [M.sector(), M.sector(sz2=1), M.sector(n=3), M.sector(nup=2, ndn=1)][seed % 4] if model != M.HUBBARD \
        else M.sector(nup=2, ndn=2)
    a, b = OHam(oracle, model, N, sector, terms), OHam(ref, model, N, sector, terms)
    assert np.array_equal(a.states(), b.states())
    for u, v in zip(a.csr(), b.csr()):
        assert np.array_equal(u, v)
