// extern "C" access to the reference qkrylov FP64 engine, compiled from the
// reference sources where they lie (recipe: oracle/Makefile, output
// oracle/_ref/libqkref.so).  Test infrastructure only: it is how the oracle
// restatement (oracle/qko.cpp) is pinned to the real reference and how the
// golden fixtures under tests/golden/ are produced.  It exists only in the
// build container that holds the reference sources.
//
// The reference keeps its CSR private (include/qkrylov/hamiltonian/
// matrix_free_hamiltonian.hpp:67-71); to dump the generated matrix entries in
// the reference's own order this translation unit opens the class up.
// ftlm.cpp is included here (and not compiled separately) to reach its
// anonymous-namespace helpers compute_tridiag / diagonalize_tridiag_components
// (src/solvers/ftlm.cpp:24,61).
#ifndef QKRYLOV_DOUBLE_PRECISION
#define QKRYLOV_DOUBLE_PRECISION
#endif
#include <algorithm>
#include <complex>
#include <cstdint>
#include <cstring>
#include <memory>
#include <random>
#include <string>
#include <vector>
#include <unordered_map>
#include <stdexcept>
#define private public
#include "qkrylov/hamiltonian/matrix_free_hamiltonian.hpp"
#undef private
#include "qkrylov/basis/spinhalf_basis.hpp"
#include "qkrylov/basis/fermion_basis.hpp"
#include "qkrylov/basis/hubbard_basis.hpp"
#include "qkrylov/basis/tj_basis.hpp"
#include "qkrylov/sites/spinhalf_site.hpp"
#include "qkrylov/sites/fermion_site.hpp"
#include "qkrylov/sites/hubbard_site.hpp"
#include "qkrylov/sites/tj_site.hpp"
#include "qkrylov/solvers/lanczos.hpp"
#include "qkrylov/solvers/davidson.hpp"
#include "qkrylov/solvers/dynamics.hpp"
#include "src/solvers/ftlm.cpp"  // via -I<reference root>

using namespace qkrylov::fp64;
using HamT = MatrixFreeHamiltonian<Kokkos::DefaultExecutionSpace>;

namespace {
struct RefHandle {
    std::shared_ptr<Basis> basis;
    std::unique_ptr<HamT> H;
};
std::string g_err;
}

extern "C" {

const char* qkref64_last_error(void) { return g_err.c_str(); }

// model: 0 spin-1/2, 1 spinless fermion, 2 Hubbard, 3 t-J.
// sector: {use_sz, sz2, use_nup, nup, use_ndn, ndn, use_n, n}
// terms: n_terms terms; term t has nfac[t] factors, taken in order from the
// flattened ops[] / sites[] arrays.
void* qkref64_create(int model, int nsites, const int* sector, int n_terms,
                     const double* coeff_re, const double* coeff_im, const int* nfac,
                     const char* const* ops, const int* sites) {
    try {
        Sector sec;
        sec.use_sz = sector[0]; sec.sz2 = sector[1];
        sec.use_nup = sector[2]; sec.nup = sector[3];
        sec.use_ndn = sector[4]; sec.ndn = sector[5];
        sec.use_n = sector[6]; sec.n = sector[7];
        auto h = std::make_unique<RefHandle>();
        std::shared_ptr<Site> site;
        switch (model) {
            case 0: h->basis = std::make_shared<SpinHalfBasis>(nsites, sec); site = std::make_shared<SpinHalfSite>(); break;
            case 1: h->basis = std::make_shared<FermionBasis>(nsites, sec); site = std::make_shared<FermionSite>(); break;
            case 2: h->basis = std::make_shared<HubbardBasis>(nsites, sec); site = std::make_shared<HubbardSite>(); break;
            case 3: h->basis = std::make_shared<TJBasis>(nsites, sec); site = std::make_shared<TJSite>(); break;
            default: g_err = "bad model"; return nullptr;
        }
        OpSum os;
        int k = 0;
        for (int t = 0; t < n_terms; ++t) {
            OperatorTerm term;
            term.coeff = Complex(coeff_re[t], coeff_im[t]);
            for (int f = 0; f < nfac[t]; ++f, ++k) term.factors.push_back({std::string(ops[k]), sites[k]});
            os.add_term(term);
        }
        h->H = std::make_unique<HamT>(h->basis, site, os);
        return h.release();
    } catch (const std::exception& e) {
        g_err = e.what();
        return nullptr;
    }
}

void qkref64_destroy(void* hp) { delete static_cast<RefHandle*>(hp); }

uint64_t qkref64_dim(void* hp) { return static_cast<RefHandle*>(hp)->H->dimension(); }

void qkref64_states(void* hp, uint64_t* out) {
    auto* h = static_cast<RefHandle*>(hp);
    for (uint64_t i = 0; i < h->basis->size(); ++i) out[i] = h->basis->state(i);
}

int64_t qkref64_index(void* hp, uint64_t s) {
    auto* h = static_cast<RefHandle*>(hp);
    if (!h->basis->contains(s)) return -1;
    return (int64_t)h->basis->index(s);
}

uint64_t qkref64_nnz(void* hp) {
    auto* h = static_cast<RefHandle*>(hp);
    return h->H->col_indices_.extent(0);
}

// CSR in the reference's order: row_offsets[dim+1], cols[nnz], vals[2*nnz].
void qkref64_csr(void* hp, int32_t* row_offsets, int32_t* cols, double* vals) {
    auto* h = static_cast<RefHandle*>(hp);
    const auto& H = *h->H;
    const uint64_t dim = H.dimension();
    for (uint64_t i = 0; i <= dim; ++i) row_offsets[i] = H.row_offsets_(i);
    const uint64_t nnz = H.col_indices_.extent(0);
    for (uint64_t j = 0; j < nnz; ++j) {
        cols[j] = H.col_indices_(j);
        vals[2 * j] = H.values_(j).real();
        vals[2 * j + 1] = H.values_(j).imag();
    }
}

void qkref64_apply(void* hp, const double* x, double* y) {
    auto* h = static_cast<RefHandle*>(hp);
    h->H->apply(reinterpret_cast<const Complex*>(x), reinterpret_cast<Complex*>(y));
}

void qkref64_diagonal(void* hp, double* d) {
    auto* h = static_cast<RefHandle*>(hp);
    auto v = h->H->diagonal_host();
    for (size_t i = 0; i < v.size(); ++i) { d[2 * i] = v[i].real(); d[2 * i + 1] = v[i].imag(); }
}

int qkref64_lanczos(void* hp, int maxiter, double tol, double* energy, int* iters, int* conv, double* evec) {
    try {
        auto* h = static_cast<RefHandle*>(hp);
        auto r = lanczos_ground_state(*h->H, maxiter, tol);
        *energy = r.energy; *iters = r.iterations; *conv = r.converged ? 1 : 0;
        if (evec) for (size_t i = 0; i < r.eigenvector.size(); ++i) { evec[2 * i] = r.eigenvector[i].real(); evec[2 * i + 1] = r.eigenvector[i].imag(); }
        return 0;
    } catch (const std::exception& e) { g_err = e.what(); return -2; }
}

int qkref64_davidson(void* hp, int n_eig, int max_sub, double tol, double* evals, double* evecs, int* iters, int* conv, int* n_out) {
    try {
        auto* h = static_cast<RefHandle*>(hp);
        auto r = davidson_lowest(*h->H, n_eig, max_sub, tol);
        const uint64_t dim = h->H->dimension();
        *iters = r.iterations; *conv = r.converged ? 1 : 0; *n_out = (int)r.eigenvalues.size();
        for (size_t k = 0; k < r.eigenvalues.size(); ++k) {
            evals[k] = r.eigenvalues[k];
            if (evecs) for (uint64_t i = 0; i < dim; ++i) {
                evecs[k * 2 * dim + 2 * i] = r.eigenvectors[k][i].real();
                evecs[k * 2 * dim + 2 * i + 1] = r.eigenvectors[k][i].imag();
            }
        }
        return 0;
    } catch (const std::exception& e) { g_err = e.what(); return -2; }
}

int qkref64_cf(void* hp, const double* phi0, int n_iter, double* alphas, double* betas, double* norm, int* n_alpha, int* n_beta) {
    try {
        auto* h = static_cast<RefHandle*>(hp);
        const uint64_t dim = h->H->dimension();
        HostVector p(dim);
        for (uint64_t i = 0; i < dim; ++i) p[i] = Complex(phi0[2 * i], phi0[2 * i + 1]);
        auto r = continued_fraction_coeffs(*h->H, p, n_iter);
        *norm = r.norm_phi0; *n_alpha = (int)r.alphas.size(); *n_beta = (int)r.betas.size();
        for (size_t i = 0; i < r.alphas.size(); ++i) alphas[i] = r.alphas[i];
        for (size_t i = 0; i < r.betas.size(); ++i) betas[i] = r.betas[i];
        return 0;
    } catch (const std::exception& e) { g_err = e.what(); return -2; }
}

double qkref64_spectral(const double* alphas, const double* betas, size_t n, double norm, double omega, double E0, double eta) {
    return evaluate_spectral_function(alphas, betas, n, norm, omega, E0, eta);
}

int qkref64_ftlm(void* hp, double beta, int n_random, int n_steps, double* Z, double* E, double* Cv) {
    try {
        auto* h = static_cast<RefHandle*>(hp);
        auto r = ftlm(*h->H, beta, n_random, n_steps);
        *Z = r.partition_function; *E = r.internal_energy; *Cv = r.specific_heat;
        return 0;
    } catch (const std::exception& e) { g_err = e.what(); return -2; }
}

// The FTLM tridiagonals of the reference's own random vectors (mt19937(42),
// src/solvers/ftlm.cpp:133-148), so Z/E/Cv can be evaluated at many beta.
// alphas/betas: n_random * n_steps each (row r holds vector r), counts per row.
int qkref64_ftlm_tridiag(void* hp, int n_random, int n_steps, double* alphas, double* betas,
                         int* n_alpha, int* n_beta, double* norms) {
    try {
        auto* h = static_cast<RefHandle*>(hp);
        const Index dim = h->H->dimension();
        std::mt19937 rng(42);
        std::normal_distribution<Real> dist(0.0, 1.0);
        for (int r = 0; r < n_random; ++r) {
            VectorView<Kokkos::DefaultExecutionSpace> r_vec("r_vec", dim);
            auto rh = Kokkos::create_mirror_view(r_vec);
            for (Index i = 0; i < dim; ++i) rh(i) = KComplex(dist(rng), dist(rng));
            Kokkos::deep_copy(r_vec, rh);
            norms[r] = norm(r_vec);
            auto td = compute_tridiag(*h->H, r_vec, n_steps);
            n_alpha[r] = (int)td.alphas.size(); n_beta[r] = (int)td.betas.size();
            for (size_t i = 0; i < td.alphas.size(); ++i) alphas[(size_t)r * n_steps + i] = td.alphas[i];
            for (size_t i = 0; i < td.betas.size(); ++i) betas[(size_t)r * n_steps + i] = td.betas[i];
        }
        return 0;
    } catch (const std::exception& e) { g_err = e.what(); return -2; }
}

// Eigenvalues and first components of a tridiagonal, by the reference's own
// routine (src/solvers/ftlm.cpp:61-119).
void qkref64_tridiag_components(const double* a, const double* b, int n, double* evals, double* first) {
    std::vector<Real> av(a, a + n), bv(b, b + (n > 0 ? n - 1 : 0));
    auto r = diagonalize_tridiag_components(av, bv);
    for (size_t i = 0; i < r.eigenvalues.size(); ++i) { evals[i] = r.eigenvalues[i]; first[i] = r.first_components[i]; }
}

}  // extern "C"
