/* Oracle restatement of qkrylov's hot path (CPU, test infrastructure only).
 *
 * This is the checker for the GPU library: tests, __graft_entry__.smoke() and
 * bench.py's CPU baseline are the only callers.  The product library never
 * links or loads it.  It restates, in plain C++ over std::complex<double>, the
 * reference's basis enumeration, site actions, CSR assembly, CSR apply, BLAS-1,
 * Lanczos, Davidson, continued fraction and FTLM (each function cites the
 * reference file:line it follows), and it is pinned against the reference
 * itself (oracle/_ref, built by oracle/Makefile) and against the golden
 * fixtures in tests/golden/.
 *
 * Conventions shared with oracle/ref_capi64.cpp:
 *   model  : 0 spin-1/2, 1 spinless fermion, 2 Hubbard, 3 t-J
 *   sector : int[8] = {use_sz, sz2, use_nup, nup, use_ndn, ndn, use_n, n}
 *   terms  : n_terms, coeff_re[t], coeff_im[t], nfac[t], then the factors of
 *            all terms flattened in order in ops[] / sites[].
 *   vectors: interleaved complex doubles [re, im, re, im, ...].
 */
#ifndef QKO_H
#define QKO_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

const char* qko_last_error(void);
void*    qko_create(int model, int nsites, const int* sector, int n_terms, const double* coeff_re,
                    const double* coeff_im, const int* nfac, const char* const* ops, const int* sites);
/* Basis only (no CSR); for state/index checks at sizes where a CSR is too big. */
void*    qko_basis_create(int model, int nsites, const int* sector);
void     qko_destroy(void* h);
uint64_t qko_dim(void* h);
void     qko_states(void* h, uint64_t* out);
int64_t  qko_index(void* h, uint64_t s);
uint64_t qko_nnz(void* h);
void     qko_csr(void* h, int32_t* row_offsets, int32_t* cols, double* vals);
void     qko_apply(void* h, const double* x, double* y);
void     qko_diagonal(void* h, double* d);
int      qko_lanczos(void* h, int maxiter, double tol, double* energy, int* iters, int* conv, double* evec);
/* Lanczos exactly as qko_lanczos but from a caller-given start vector (normalised inside). */
int      qko_lanczos_from(void* h, const double* v0, int maxiter, double tol, double* energy, int* iters,
                          int* conv, double* evec, double* alphas, double* betas);
int      qko_davidson(void* h, int n_eig, int max_sub, double tol, double* evals, double* evecs, int* iters,
                      int* conv, int* n_out);
/* qko_davidson with the iteration cap max_iter in place of the reference's 100. */
int      qko_davidson_max(void* h, int n_eig, int max_sub, double tol, int max_iter, double* evals, double* evecs,
                          int* iters, int* conv, int* n_out);
int      qko_cf(void* h, const double* phi0, int n_iter, double* alphas, double* betas, double* norm,
                int* n_alpha, int* n_beta);
double   qko_spectral(const double* alphas, const double* betas, size_t n, double norm, double omega,
                      double E0, double eta);
int      qko_ftlm(void* h, double beta, int n_random, int n_steps, double* Z, double* E, double* Cv);
int      qko_ftlm_tridiag(void* h, int n_random, int n_steps, double* alphas, double* betas, int* n_alpha,
                          int* n_beta, double* norms);
void     qko_tridiag_components(const double* a, const double* b, int n, double* evals, double* first);
double   qko_tridiag_ground(const double* a, const double* b, int n, double* evec);
/* Reference random streams (libstdc++ mt19937 + distributions, draw order as the
 * reference binary built with g++ evaluates KComplex(dist(rng), dist(rng))). */
void     qko_rng_uniform_complex(uint32_t seed, uint64_t n, double* out);
void     qko_rng_normal_complex(uint32_t seed, uint64_t n, double* out);

/* Host threads the oracle's OpenMP loops use from now on (n > 0). */
void     qko_set_threads(int n);
/* qko_create with the CSR of every row built by all host threads (same CSR,
 * same entry order); for the CPU baseline at full size. */
void*    qko_create_parallel(int model, int nsites, const int* sector, int n_terms, const double* coeff_re,
                             const double* coeff_im, const int* nfac, const char* const* ops, const int* sites);
/* The reference's Lanczos (full reorthogonalisation, tridiagonal ground state
 * every step) for exactly n_steps steps, from v0 (interleaved complex, not
 * normalised) or, with v0 NULL, from the reference's mt19937(1234) start
 * vector; the wall time of every step is written to step_seconds[*n_done]
 * (the Ritz vector at the end is not timed). */
int      qko_lanczos_timed(void* h, const double* v0, int n_steps, double* step_seconds, int* n_done,
                           double* energy);

/* CPU baseline: the reference algorithm (host CSR + CSR gather + full
 * reorthogonalisation) timed on a bounded sample of rows.  Builds the CSR of
 * rows [row0, row0+nrows) only. */
void*    qko_sample_create(int model, int nsites, const int* sector, int n_terms, const double* coeff_re,
                           const double* coeff_im, const int* nfac, const char* const* ops, const int* sites,
                           uint64_t row0, uint64_t nrows);
/* Time `reps` CSR applies of the sampled rows (x of full dimension) and `reps`
 * rounds of `k_reorth` dot+axpy pairs plus the 3-term update over the sampled
 * length.  Returns seconds per apply and per vector-algebra round. */
int      qko_sample_time(void* h, int reps, int k_reorth, int n_threads, double* t_apply, double* t_vec);

#ifdef __cplusplus
}
#endif
#endif
