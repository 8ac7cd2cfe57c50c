/* A plain C11 caller of the library's C ABI, compiled and linked against
 * include/qkrylov/c_api.h and libqkrylov_gb300.so the way a foreign-language
 * binding would be: the sector -> basis -> site -> opsum -> hamiltonian ->
 * apply -> Lanczos -> Davidson -> continued fraction -> FTLM flow of the
 * reference's own C API test (tests/test_c_api.cpp:19-149), on the periodic
 * Heisenberg chain L=10, Sz=0 (dim 252).  It checks what can be checked
 * without a reference value (agreement of the float and FP64 paths, H psi =
 * E psi, norms, signs) and prints the energies for the caller to compare with
 * the reference's.  Exit status 0 when every check holds. */
#include "qkrylov/c_api.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#define CHECK(cond)                                                     \
    do {                                                                \
        if (!(cond)) {                                                  \
            fprintf(stderr, "check failed at line %d: %s\n", __LINE__, #cond); \
            return 1;                                                   \
        }                                                               \
    } while (0)

enum { N = 10 };

int main(void) {
    qkrylov_sector_h sec = qkrylov_sector_create();
    CHECK(sec != NULL);
    CHECK(qkrylov_sector_set_sz(sec, 0) == QKRYLOV_SUCCESS);
    qkrylov_basis_h basis = qkrylov_spinhalf_basis_create(N, sec);
    CHECK(basis != NULL);
    const uint64_t dim = qkrylov_basis_dimension(basis);
    CHECK(dim == 252);
    CHECK(qkrylov_basis_nsites(basis) == N);
    for (uint64_t i = 0; i < dim; ++i) {
        const uint64_t s = qkrylov_basis_state(basis, i);
        CHECK(qkrylov_basis_contains(basis, s) == 1);
        CHECK(qkrylov_basis_index(basis, s) == (int64_t)i);
        if (i) CHECK(s > qkrylov_basis_state(basis, i - 1));  /* ascending, as the reference orders it */
    }
    CHECK(qkrylov_basis_index(basis, 1) == -1);  /* one up spin: not in Sz = 0 */

    qkrylov_site_h site = qkrylov_spinhalf_site_create();
    CHECK(site != NULL);
    qkrylov_opsum_h ops = qkrylov_opsum_create();
    CHECK(ops != NULL);
    for (int i = 0; i < N; ++i) {
        const int j = (i + 1) % N;
        CHECK(qkrylov_opsum_add_term_2body(ops, 1.0f, 0.0f, "Sz", i, "Sz", j) == QKRYLOV_SUCCESS);
        CHECK(qkrylov_opsum_add_term_2body(ops, 0.5f, 0.0f, "Sp", i, "Sm", j) == QKRYLOV_SUCCESS);
        CHECK(qkrylov_opsum_add_term_2body(ops, 0.5f, 0.0f, "Sm", i, "Sp", j) == QKRYLOV_SUCCESS);
    }
    qkrylov_hamiltonian_h H = qkrylov_hamiltonian_create(basis, site, ops);
    CHECK(H != NULL);
    qkrylov_opsum_destroy(ops);  /* the Hamiltonian keeps its own copy of the terms */
    CHECK(qkrylov_hamiltonian_dimension(H) == dim);

    float* xr = calloc(dim, sizeof(float));
    float* xi = calloc(dim, sizeof(float));
    float* yr = calloc(dim, sizeof(float));
    float* yi = calloc(dim, sizeof(float));
    float* xc = calloc(2 * dim, sizeof(float));
    float* yc = calloc(2 * dim, sizeof(float));
    float* diag = calloc(dim, sizeof(float));
    float* psi = calloc(2 * dim, sizeof(float));
    double* psi64 = calloc(2 * dim, sizeof(double));
    float* hv = calloc(2 * dim, sizeof(float));
    CHECK(xr && xi && yr && yi && xc && yc && diag && psi && psi64 && hv);
    for (uint64_t i = 0; i < dim; ++i) {
        xr[i] = (float)(0.25 + 0.001 * (double)i);
        xi[i] = (float)(-0.5 + 0.002 * (double)i);
        xc[2 * i] = xr[i];
        xc[2 * i + 1] = xi[i];
    }
    CHECK(qkrylov_hamiltonian_apply(H, xr, xi, yr, yi) == QKRYLOV_SUCCESS);
    CHECK(qkrylov_hamiltonian_apply_complex(H, xc, yc) == QKRYLOV_SUCCESS);
    for (uint64_t i = 0; i < dim; ++i) {
        CHECK(fabsf(yc[2 * i] - yr[i]) <= 1e-6f * (1.0f + fabsf(yr[i])));
        CHECK(fabsf(yc[2 * i + 1] - yi[i]) <= 1e-6f * (1.0f + fabsf(yi[i])));
    }
    CHECK(qkrylov_hamiltonian_diagonal(H, diag) == QKRYLOV_SUCCESS);
    for (uint64_t i = 0; i < dim; ++i) CHECK(fabsf(diag[i]) <= 2.5f);  /* |<Sz Sz>| sum over 10 bonds */

    qkrylov_lanczos_result_c_t lz;
    CHECK(qkrylov_lanczos_ground_state_complex(H, 200, 1e-12f, &lz, psi) == QKRYLOV_SUCCESS);
    CHECK(lz.converged == 1);
    double nrm = 0.0;
    for (uint64_t i = 0; i < 2 * dim; ++i) nrm += (double)psi[i] * psi[i];
    CHECK(fabs(nrm - 1.0) < 1e-4);

    qkrylov_lanczos_result_f64_t lz64;
    CHECK(qkrylov_lanczos_ground_state_f64(H, 300, 1e-12, NULL, &lz64, psi64) == QKRYLOV_SUCCESS);
    CHECK(fabs(lz64.energy - (double)lz.energy) < 1e-5);

    enum { K = 2 };
    float ev[K];
    float* evecs = calloc((size_t)K * 2 * dim, sizeof(float));
    CHECK(evecs != NULL);
    qkrylov_davidson_result_c_t dinfo;
    CHECK(qkrylov_davidson_lowest_complex(H, K, 20, 1e-6f, ev, evecs, &dinfo) == QKRYLOV_SUCCESS);
    CHECK(dinfo.converged == 1);
    CHECK(fabs((double)ev[0] - lz64.energy) < 1e-4);
    CHECK(ev[0] <= ev[1]);
    for (int k = 0; k < K; ++k) {
        const float* v = evecs + (size_t)k * 2 * dim;
        CHECK(qkrylov_hamiltonian_apply_complex(H, v, hv) == QKRYLOV_SUCCESS);
        for (uint64_t i = 0; i < 2 * dim; ++i) CHECK(fabsf(hv[i] - ev[k] * v[i]) < 1e-3f);
    }

    enum { NIT = 20 };
    float al[NIT], be[NIT], nphi = 0.0f;
    int ncoef = 0;
    CHECK(qkrylov_continued_fraction_coeffs_complex(H, psi, NIT, al, be, &nphi, &ncoef) == QKRYLOV_SUCCESS);
    CHECK(ncoef > 0);
    CHECK(fabsf(nphi - 1.0f) < 1e-3f);
    CHECK(fabsf(al[0] - lz.energy) < 1e-4f);  /* <psi0|H|psi0> = E0 */
    const float S = qkrylov_evaluate_spectral_function(al, be, (size_t)ncoef, nphi, 0.5f, lz.energy, 0.1f);
    CHECK(S > 0.0f);

    qkrylov_ftlm_result_c_t fr;
    CHECK(qkrylov_ftlm(H, 1.0f, 10, 20, &fr) == QKRYLOV_SUCCESS);
    CHECK(fr.partition_function > 0.0f);

    /* invalid arguments: reference status codes */
    CHECK(qkrylov_hamiltonian_apply(NULL, xr, xi, yr, yi) == QKRYLOV_ERROR_INVALID_ARG);
    CHECK(qkrylov_hamiltonian_create(NULL, site, NULL) == NULL);

    printf("E0_float %.9g\nE0_f64 %.17g\nE1_davidson %.9g\nS_0.5 %.9g\nZ_ftlm %.9g\n", (double)lz.energy,
           lz64.energy, (double)ev[1], (double)S, (double)fr.partition_function);

    qkrylov_hamiltonian_destroy(H);
    qkrylov_site_destroy(site);
    qkrylov_basis_destroy(basis);
    qkrylov_sector_destroy(sec);
    free(xr); free(xi); free(yr); free(yi); free(xc); free(yc); free(diag); free(psi); free(psi64); free(hv); free(evecs);
    return 0;
}
