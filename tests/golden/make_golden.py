"""Generate the golden fixtures in tests/golden/ from the reference itself.

Runs the reference qkrylov sources compiled unchanged by ``make -C oracle ref``
(oracle/_ref/libqkref.so, FP64 engine) on small models of every site type and
records what they produce: basis states, the CSR content (column order and
values per row), y = Hx for a seeded x, the diagonal, Lanczos/Davidson results,
continued-fraction coefficients and FTLM tridiagonals and observables.
The reference C API (FP32 engine, src/c_api.cpp) is also run on the 4-site
chain of tests/test_c_api.cpp.

Needs the reference source tree at build time; the fixtures it writes are
self-contained.  Run from the repository root:
    make -C oracle ref && OMP_NUM_THREADS=1 python tests/golden/make_golden.py
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
import models as M  # noqa: E402
from oracle_ctypes import OHam, Oracle  # noqa: E402

CASES = {
    "heis_L10_pbc_sz0": M.heisenberg(10, True, 0),
    "heis_L16_obc_sz0": M.heisenberg(16, False, 0),
    "heis_L9_obc_full": M.heisenberg(9, False, None),
    "xyz_L8_full": (M.SPIN, 8, M.sector(), M.xyz_field_terms(8, True)),
    "xyz_L8_sz0": (M.SPIN, 8, M.sector(sz2=0), M.xyz_field_terms(8, True)),
    "ferm_L10_n4": (M.FERMION, 10, M.sector(n=4), M.fermion_chain_terms(10, True)),
    "ferm_L8_full": (M.FERMION, 8, M.sector(), M.fermion_chain_terms(8, False)),
    "hub_L6_n33": M.hubbard(6, True, 3, 3),
    "hub_L5_up2": (M.HUBBARD, 5, M.sector(nup=2), M.hubbard_terms(5, True)),
    "hub_L4_full": (M.HUBBARD, 4, M.sector(), M.hubbard_terms(4, False)),
    "tj_L6_n22": (M.TJ, 6, M.sector(nup=2, ndn=2), M.tj_terms(6, True)),
    "tj_L5_full": (M.TJ, 5, M.sector(), M.tj_terms(5, False)),
}
BETAS = np.array([0.1, 1.0, 5.0])
FTLM_R, FTLM_M = 4, 20


def terms_arrays(terms):
    coeff = np.array([complex(t[0]) for t in terms], dtype=np.complex128)
    nfac = np.array([len(t[1]) for t in terms], dtype=np.int32)
    ops = np.array([f[0] for t in terms for f in t[1]])
    sites = np.array([f[1] for t in terms for f in t[1]], dtype=np.int32)
    return coeff, nfac, ops, sites


def gen_case(ref, name, model, N, sector, terms):
    h = OHam(ref, model, N, sector, terms)
    d = {}
    d["model"], d["nsites"], d["sector"] = model, N, np.array(sector, dtype=np.int32)
    d["coeff"], d["nfac"], d["ops"], d["sites"] = terms_arrays(terms)
    d["dim"] = h.dim
    d["states"] = h.states()
    if h.dim <= 5000:
        ro, cols, vals = h.csr()
        d["csr_ro"], d["csr_cols"], d["csr_vals"] = ro, cols, vals
    rng = np.random.default_rng(12345)
    x = rng.normal(size=h.dim) + 1j * rng.normal(size=h.dim)
    d["x"], d["y"] = x, h.apply(x)
    d["diag"] = h.diagonal()
    e, it, cv, v = h.lanczos(300, 1e-12, want_vec=True)
    d["lanczos_E0"], d["lanczos_iters"], d["lanczos_conv"], d["lanczos_vec"] = e, it, cv, v
    ev, it, cv, _ = h.davidson(min(3, h.dim), 20, 1e-8)
    d["davidson_evals"], d["davidson_iters"], d["davidson_conv"] = ev, it, cv
    phi0 = rng.normal(size=h.dim) + 1j * rng.normal(size=h.dim)
    a, b, nrm = h.cf(phi0, 30)
    d["cf_phi0"], d["cf_alphas"], d["cf_betas"], d["cf_norm"] = phi0, a, b, nrm
    ta, tb, na, nb, nr = h.ftlm_tridiag(FTLM_R, FTLM_M)
    d["ftlm_alphas"], d["ftlm_betas"], d["ftlm_na"], d["ftlm_nb"], d["ftlm_norms"] = ta, tb, na, nb, nr
    d["ftlm_betas_T"] = BETAS
    d["ftlm_obs"] = np.array([h.ftlm(bt, FTLM_R, FTLM_M) for bt in BETAS])
    if name == "heis_L16_obc_sz0":  # the L=16 open-chain Lanczos case: keep its fixture light
        for k in ("csr_ro", "csr_cols", "csr_vals", "x", "y", "cf_phi0", "lanczos_vec"):
            d.pop(k, None)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
    return h.dim


def gen_capi(path):
    """tests/test_c_api.cpp's 4-site chain through the reference C API (FP32 engine)."""
    L = ctypes.CDLL(path)
    vp = ctypes.c_void_p
    for f in ("qkrylov_sector_create", "qkrylov_spinhalf_basis_create", "qkrylov_spinhalf_site_create",
              "qkrylov_opsum_create", "qkrylov_hamiltonian_create"):
        getattr(L, f).restype = vp
    L.qkrylov_spinhalf_basis_create.argtypes = [ctypes.c_int, vp]
    L.qkrylov_sector_set_sz.argtypes = [vp, ctypes.c_int]
    L.qkrylov_opsum_add_term_2body.argtypes = [vp, ctypes.c_float, ctypes.c_float, ctypes.c_char_p, ctypes.c_int,
                                               ctypes.c_char_p, ctypes.c_int]
    L.qkrylov_hamiltonian_create.argtypes = [vp, vp, vp]
    L.qkrylov_hamiltonian_dimension.restype = ctypes.c_uint64
    L.qkrylov_hamiltonian_dimension.argtypes = [vp]
    fp = ctypes.POINTER(ctypes.c_float)
    L.qkrylov_hamiltonian_apply_complex.argtypes = [vp, fp, fp]

    class LR(ctypes.Structure):
        _fields_ = [("energy", ctypes.c_float), ("iterations", ctypes.c_int), ("converged", ctypes.c_int)]

    class DR(ctypes.Structure):
        _fields_ = [("iterations", ctypes.c_int), ("converged", ctypes.c_int)]

    class FR(ctypes.Structure):
        _fields_ = [("beta", ctypes.c_float), ("Z", ctypes.c_float), ("E", ctypes.c_float), ("C", ctypes.c_float)]

    L.qkrylov_lanczos_ground_state_complex.argtypes = [vp, ctypes.c_int, ctypes.c_float, ctypes.POINTER(LR), fp]
    L.qkrylov_davidson_lowest_complex.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_float, fp, fp,
                                                  ctypes.POINTER(DR)]
    L.qkrylov_continued_fraction_coeffs_complex.argtypes = [vp, fp, ctypes.c_int, fp, fp, fp,
                                                            ctypes.POINTER(ctypes.c_int)]
    L.qkrylov_evaluate_spectral_function.restype = ctypes.c_float
    L.qkrylov_evaluate_spectral_function.argtypes = [fp, fp, ctypes.c_size_t] + [ctypes.c_float] * 4
    L.qkrylov_ftlm.argtypes = [vp, ctypes.c_float, ctypes.c_int, ctypes.c_int, ctypes.POINTER(FR)]
    sec = L.qkrylov_sector_create()
    L.qkrylov_sector_set_sz(sec, 0)
    basis = L.qkrylov_spinhalf_basis_create(4, sec)
    site = L.qkrylov_spinhalf_site_create()
    op = L.qkrylov_opsum_create()
    for i in range(3):
        L.qkrylov_opsum_add_term_2body(op, 1.0, 0.0, b"Sz", i, b"Sz", i + 1)
        L.qkrylov_opsum_add_term_2body(op, 0.5, 0.0, b"Sp", i, b"Sm", i + 1)
        L.qkrylov_opsum_add_term_2body(op, 0.5, 0.0, b"Sm", i, b"Sp", i + 1)
    H = L.qkrylov_hamiltonian_create(basis, site, op)
    dim = L.qkrylov_hamiltonian_dimension(H)
    x = np.ones(2 * dim, dtype=np.float32)
    x[1::2] = 0
    y = np.zeros(2 * dim, dtype=np.float32)
    L.qkrylov_hamiltonian_apply_complex(H, x.ctypes.data_as(fp), y.ctypes.data_as(fp))
    lr = LR()
    psi = np.zeros(2 * dim, dtype=np.float32)
    L.qkrylov_lanczos_ground_state_complex(H, 200, 1e-12, ctypes.byref(lr), psi.ctypes.data_as(fp))
    ev = np.zeros(2, dtype=np.float32)
    evec = np.zeros(4 * dim, dtype=np.float32)
    dr = DR()
    L.qkrylov_davidson_lowest_complex(H, 2, 20, 1e-6, ev.ctypes.data_as(fp), evec.ctypes.data_as(fp), ctypes.byref(dr))
    a = np.zeros(20, dtype=np.float32)
    b = np.zeros(20, dtype=np.float32)
    nrm = np.zeros(1, dtype=np.float32)
    nc = ctypes.c_int()
    L.qkrylov_continued_fraction_coeffs_complex(H, psi.ctypes.data_as(fp), 20, a.ctypes.data_as(fp), b.ctypes.data_as(fp),
                                                nrm.ctypes.data_as(fp), ctypes.byref(nc))
    s05 = L.qkrylov_evaluate_spectral_function(a.ctypes.data_as(fp), b.ctypes.data_as(fp), nc.value, float(nrm[0]), 0.5,
                                               lr.energy, 0.1)
    fr = FR()
    L.qkrylov_ftlm(H, 1.0, 10, 20, ctypes.byref(fr))
    np.savez_compressed(os.path.join(HERE, "capi_heis4.npz"), dim=dim, y=y, energy=lr.energy, iters=lr.iterations,
                        conv=lr.converged, psi=psi, dav_evals=ev, dav_iters=dr.iterations, dav_conv=dr.converged,
                        cf_alphas=a[: nc.value], cf_betas=b[: nc.value], cf_norm=nrm[0], s05=s05,
                        ftlm=np.array([fr.beta, fr.Z, fr.E, fr.C]))


def main():
    os.environ.setdefault("OMP_NUM_THREADS", "1")
    ref = Oracle("qkref64")
    for name, (model, N, sector, terms) in CASES.items():
        dim = gen_case(ref, name, model, N, sector, terms)
        print(f"{name}: dim {dim}")
    gen_capi(ref.lib._name)
    print("capi_heis4")


if __name__ == "__main__":
    main()
