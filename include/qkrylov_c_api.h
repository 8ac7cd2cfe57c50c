/* qkrylov C ABI, served by libqkrylov_gb300.so (GB300 / sm_103a).
 *
 * Part 1 declares every symbol of the reference C API with the reference's
 * names, argument meaning, float signatures and status codes
 * (qkrylov: include/qkrylov/c_api.h:14-168, implemented in src/c_api.cpp);
 * existing callers (the Julia binding's ccall table in bindings/julia/src,
 * or any FFI) relink against this library unchanged.  The float entry points
 * run the FP64 GPU engine and cast results to float (the reference compiles
 * its C API into its FP32 engine, CMakeLists.txt:47).
 *
 * Part 2 adds what the float ABI cannot carry: FP64 twins (suffix _f64), the
 * mixed-precision and batched solver forms, device-pointer variants for
 * callers whose vectors already live on the GPU, an error-string getter and
 * a debug dump of the generated matrix entries.
 *
 * Vectors are complex, interleaved [re, im, re, im, ...], in the reference's
 * basis order (ascending state integers; Hubbard/t-J states interleaved with
 * the up electron of site i at bit 2i and the down electron at bit 2i+1).
 * Every call is synchronous.  A handle is not safe for concurrent use from
 * several threads; distinct handles are.
 */
#ifndef QKRYLOV_GB300_C_API_H
#define QKRYLOV_GB300_C_API_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status codes */
/* c_api.h:14-16 */
#define QKRYLOV_SUCCESS                0
#define QKRYLOV_ERROR_INVALID_ARG     -1
#define QKRYLOV_ERROR_EXCEPTION       -2
/* additions: a CUDA runtime error (message in qkrylov_last_error()), and a
 * bounded device-side wait that gave up */
#define QKRYLOV_ERROR_CUDA            -3
#define QKRYLOV_ERROR_DEVICE_TIMEOUT  -4

/* ---------------------------------------------------------------- handles (c_api.h:21-25) */
typedef struct qkrylov_sector_t*      qkrylov_sector_h;
typedef struct qkrylov_basis_t*       qkrylov_basis_h;
typedef struct qkrylov_site_t*        qkrylov_site_h;
typedef struct qkrylov_opsum_t*       qkrylov_opsum_h;
typedef struct qkrylov_hamiltonian_t* qkrylov_hamiltonian_h;

/* ================================================================ Part 1: reference ABI */

/* Sector API (c_api.h:30-39) */
qkrylov_sector_h qkrylov_sector_create(void);
void             qkrylov_sector_destroy(qkrylov_sector_h sector);
int              qkrylov_sector_set_sz(qkrylov_sector_h sector, int sz2);
int              qkrylov_sector_set_hubbard_particles(qkrylov_sector_h sector, int nup, int ndn);
int              qkrylov_sector_set_n(qkrylov_sector_h sector, int n);
int              qkrylov_sector_set_nb(qkrylov_sector_h sector, int nb);
int              qkrylov_sector_get_sz(qkrylov_sector_h sector, int* sz2_out, int* active_out);
int              qkrylov_sector_get_hubbard_particles(qkrylov_sector_h sector, int* nup_out, int* ndn_out, int* active_out);
int              qkrylov_sector_get_n(qkrylov_sector_h sector, int* n_out, int* active_out);
int              qkrylov_sector_get_nb(qkrylov_sector_h sector, int* nb_out, int* active_out);

/* Basis API (c_api.h:44-53).  Bases are built on the host from combinatorial
 * tables; no GPU is needed until a Hamiltonian is created. */
qkrylov_basis_h  qkrylov_spinhalf_basis_create(int num_sites, qkrylov_sector_h sector);
qkrylov_basis_h  qkrylov_fermion_basis_create(int num_sites, qkrylov_sector_h sector);
qkrylov_basis_h  qkrylov_hubbard_basis_create(int num_sites, qkrylov_sector_h sector);
qkrylov_basis_h  qkrylov_tj_basis_create(int num_sites, qkrylov_sector_h sector);
void             qkrylov_basis_destroy(qkrylov_basis_h basis);
uint64_t         qkrylov_basis_dimension(qkrylov_basis_h basis);
int              qkrylov_basis_nsites(qkrylov_basis_h basis);
uint64_t         qkrylov_basis_state(qkrylov_basis_h basis, uint64_t index);
int64_t          qkrylov_basis_index(qkrylov_basis_h basis, uint64_t state_bitstring);
int              qkrylov_basis_contains(qkrylov_basis_h basis, uint64_t state_bitstring);

/* Site API (c_api.h:58-62) */
qkrylov_site_h   qkrylov_spinhalf_site_create(void);
qkrylov_site_h   qkrylov_fermion_site_create(void);
qkrylov_site_h   qkrylov_hubbard_site_create(void);
qkrylov_site_h   qkrylov_tj_site_create(void);
void             qkrylov_site_destroy(qkrylov_site_h site);

/* OpSum API (c_api.h:67-76) */
qkrylov_opsum_h  qkrylov_opsum_create(void);
void             qkrylov_opsum_destroy(qkrylov_opsum_h opsum);
int              qkrylov_opsum_clear(qkrylov_opsum_h opsum);
int              qkrylov_opsum_add_term_1body(qkrylov_opsum_h opsum, float coeff_real, float coeff_imag,
                                             const char* op1, int site1);
int              qkrylov_opsum_add_term_2body(qkrylov_opsum_h opsum, float coeff_real, float coeff_imag,
                                             const char* op1, int site1,
                                             const char* op2, int site2);
int              qkrylov_opsum_add_term_nbody(qkrylov_opsum_h opsum, float coeff_real, float coeff_imag,
                                             int n_factors, const char** ops, const int* sites);

/* Matrix-free Hamiltonian API (c_api.h:81-100).  Creation compiles the OpSum
 * and uploads the basis tables to the current CUDA device; it returns NULL on
 * failure (unknown operator, site outside the site type's bit range, no GPU). */
qkrylov_hamiltonian_h qkrylov_hamiltonian_create(qkrylov_basis_h basis,
                                                qkrylov_site_h site,
                                                qkrylov_opsum_h opsum);
void                  qkrylov_hamiltonian_destroy(qkrylov_hamiltonian_h h);
uint64_t              qkrylov_hamiltonian_dimension(qkrylov_hamiltonian_h h);
int                   qkrylov_hamiltonian_apply(qkrylov_hamiltonian_h h,
                                                const float* x_real, const float* x_imag,
                                                float* y_real, float* y_imag);
int                   qkrylov_hamiltonian_apply_complex(qkrylov_hamiltonian_h h,
                                                        const float* x_complex,
                                                        float* y_complex);
int                   qkrylov_hamiltonian_diagonal(qkrylov_hamiltonian_h h,
                                                   float* diag_out);

/* Solvers API (c_api.h:105-168) */
typedef struct {
    float energy;
    int iterations;
    int converged;
} qkrylov_lanczos_result_c_t;

typedef struct {
    int iterations;
    int converged;
} qkrylov_davidson_result_c_t;

int qkrylov_lanczos_ground_state(qkrylov_hamiltonian_h h, int maxiter, float tol,
                                 qkrylov_lanczos_result_c_t* result);
int qkrylov_lanczos_ground_state_complex(qkrylov_hamiltonian_h h, int maxiter, float tol,
                                         qkrylov_lanczos_result_c_t* result, float* eigenvector_complex);
int qkrylov_davidson_lowest_complex(qkrylov_hamiltonian_h h, int n_eig, int max_subspace, float tol,
                                    float* eigenvalues_out, float* eigenvectors_complex_out,
                                    qkrylov_davidson_result_c_t* result_info);
int qkrylov_continued_fraction_coeffs_complex(qkrylov_hamiltonian_h h, const float* phi0_complex, int n_iter,
                                              float* alphas_out, float* betas_out, float* norm_phi0_out,
                                              int* num_coeffs_out);
float qkrylov_evaluate_spectral_function(const float* alphas, const float* betas, size_t n, float norm_phi0,
                                         float omega, float E0, float eta);

typedef struct {
    float beta;
    float partition_function;
    float internal_energy;
    float specific_heat;
} qkrylov_ftlm_result_c_t;

int qkrylov_ftlm(qkrylov_hamiltonian_h h, float beta, int n_random, int n_steps, qkrylov_ftlm_result_c_t* result);

/* ================================================================ Part 2: additions */

/* Message of the last failing call on this thread ("" if none). */
const char* qkrylov_last_error(void);

/* Constrain one spin species alone (the reference's C++ Sector allows it,
 * sector.hpp:24-31; its C API sets both together). */
int qkrylov_sector_set_nup(qkrylov_sector_h sector, int nup);
int qkrylov_sector_set_ndn(qkrylov_sector_h sector, int ndn);

/* OpSum term with double-precision coefficient (c_api.h:75-76 takes float). */
int qkrylov_opsum_add_term_nbody_f64(qkrylov_opsum_h opsum, double coeff_real, double coeff_imag,
                                     int n_factors, const char** ops, const int* sites);

/* FP64 twins of the apply / diagonal calls (c_api.h:89-100). */
int qkrylov_hamiltonian_apply_complex_f64(qkrylov_hamiltonian_h h, const double* x_complex, double* y_complex);
int qkrylov_hamiltonian_diagonal_f64(qkrylov_hamiltonian_h h, double* diag_out /* real parts, dim */);

/* Same, but x and y are device pointers (reference order) and the work is
 * queued on `stream` (a cudaStream_t, NULL = legacy default stream); the call
 * returns without synchronising.  The _f32 form runs the FP32 kernel.  Device
 * pointers of this section must sit on the grid of whole complex elements
 * (16 bytes for complex FP64, 8 for complex FP32), else
 * QKRYLOV_ERROR_INVALID_ARG before any launch. */
int qkrylov_hamiltonian_apply_device_f64(qkrylov_hamiltonian_h h, const void* d_x, void* d_y, void* stream);
int qkrylov_hamiltonian_apply_device_f32(qkrylov_hamiltonian_h h, const void* d_x, void* d_y, void* stream);

/* <x, y> = sum_i conj(x_i) y_i of two device vectors of n complex elements
 * (interleaved), run on `stream` (NULL = legacy default stream) on the current
 * GPU; result[0], result[1] (host) receive the real and imaginary parts, and
 * the call synchronises the stream.  The reference's dot (include/qkrylov/
 * linalg/vector_ops.hpp:14-32) returned a host scalar the same way.  The _f32
 * form reduces FP32 data with compensated (FP64-accurate) arithmetic.  Scratch
 * for the partial sums is allocated by the library on first use. */
int qkrylov_vector_dot_device_f64(const void* d_x, const void* d_y, uint64_t n, double* result, void* stream);
int qkrylov_vector_dot_device_f32(const void* d_x, const void* d_y, uint64_t n, double* result, void* stream);

/* Same result as qkrylov_vector_dot_device_f64, but the library allocates
 * nothing: no counterpart in the reference.  It is for callers that cannot let
 * a library call cudaMalloc -- applications that reserve the GPU's memory in
 * their own pool or run under a hard memory cap, and latency-critical loops
 * that cannot take cudaMalloc's implicit device synchronisation.  The partial
 * sums go to a fixed 256 KiB array compiled into the library (held by every
 * GPU that loads it until exit), so n is limited to 134,217,728 complex
 * elements; larger n returns QKRYLOV_ERROR_INVALID_ARG.  All calls share that
 * array: calls that overlap on the GPU race and must be serialised by the
 * caller.  The first call on a GPU looks up the array's address there and
 * loads the call's kernels; under CUDA's lazy module loading that is when the
 * array and the kernels take their device memory, so make one call with n = 0
 * (the warm-up: it computes nothing) before reserving the GPU's memory.  The
 * call waits for `stream` to read the result, so it cannot be used inside a
 * stream capture. */
int qkrylov_vector_dot_device_f64_noalloc(const void* d_x, const void* d_y, uint64_t n, double* result,
                                          void* stream);

/* Lanczos ground state, FP64 (reference semantics: full reorthogonalisation,
 * stop when |E_k - E_{k-1}| < tol; lanczos.cpp:101-202).  The start vector is
 * the reference's (mt19937(1234), uniform[-1,1] complex) unless v0 (dim complex,
 * reference order) is given. */
typedef struct {
    double energy;           /* reported ground-state energy */
    double energy_tridiag;   /* lowest eigenvalue of the Lanczos tridiagonal */
    double residual;         /* ||H psi - E psi|| in FP64, or -1 if not computed */
    int iterations;
    int converged;
    int selective_steps;     /* mixed form: steps re-orthogonalised against the Ritz vector */
    double seconds_loop;     /* wall time of the Lanczos loop */
    double seconds_refine;   /* wall time of the FP64 refinement (mixed form) */
    double seconds_spmv;     /* CUDA-event time of the loop's SpMV launches, summed */
    int spmv_calls;          /* SpMV launches in the loop */
} qkrylov_lanczos_result_f64_t;

int qkrylov_lanczos_ground_state_f64(qkrylov_hamiltonian_h h, int maxiter, double tol, const double* v0_complex,
                                     qkrylov_lanczos_result_f64_t* result, double* eigenvector_complex);
/* Mixed form: FP32 vectors and FP32 SpMV, compensated (FP64-accurate)
 * reductions, selective reorthogonalisation against the converged Ritz vector,
 * then one FP64 SpMV for the Rayleigh quotient and residual.  `energy` is the
 * refined value. */
int qkrylov_lanczos_ground_state_mixed(qkrylov_hamiltonian_h h, int maxiter, double tol, const double* v0_complex,
                                       qkrylov_lanczos_result_f64_t* result, double* eigenvector_complex);
/* Performance form of both: exactly n_steps steps (no early exit); mixed = 1
 * selects the mixed form, 0 the FP64 form with full reorthogonalisation and 2
 * the FP64 form with the mixed form's selective reorthogonalisation (against
 * the lowest Ritz vector once it has converged to sqrt(eps_64) ||T||).  The start vector is v0_complex (host, reference
 * order) if given, else a seeded device Gaussian (Philox4x32-10, `seed`).
 * eigenvector_complex (host, optional) receives the Ritz vector. */
int qkrylov_lanczos_fixed_steps(qkrylov_hamiltonian_h h, int n_steps, uint64_t seed, int mixed,
                                const double* v0_complex, qkrylov_lanczos_result_f64_t* result,
                                double* eigenvector_complex);
/* Lowest Ritz values of the Lanczos tridiagonal after n_steps steps from the
 * seeded Philox start of qkrylov_lanczos_fixed_steps (mixed: 0 FP64 with full
 * reorthogonalisation, 1 the mixed form, 2 FP64 with selective
 * reorthogonalisation): values[0..*n_out-1] ascending, *n_out = min(n_values,
 * steps run); selective reorthogonalisation guards the converged Ritz vectors
 * among the min(n_values, 4) lowest (the ground-state entry points guard the
 * lowest only), and *n_locked (may be NULL) = how many it held at the end (0
 * with full reorthogonalisation).  No counterpart in the reference, whose Lanczos reports
 * the ground state only (src/solvers/lanczos.cpp:175). */
int qkrylov_lanczos_ritz_values(qkrylov_hamiltonian_h h, int n_steps, uint64_t seed, int mixed, int n_values,
                                double* values, int* n_out, int* n_locked);

/* Number of kernels this library has launched so far in the process. */
uint64_t qkrylov_kernel_launches(void);

/* Bounded device-side waits (a staged SpMV waiting for its asynchronous copy)
 * that gave up on the current GPU since the process started; waits for that
 * GPU first.  Returns QKRYLOV_ERROR_DEVICE_TIMEOUT if the count is non-zero,
 * else QKRYLOV_SUCCESS.  A kernel whose wait gave up reads its operand from
 * global memory instead, so its results are complete; a solver call during
 * which the count grew returns QKRYLOV_ERROR_DEVICE_TIMEOUT. */
int qkrylov_device_wait_timeouts(uint32_t* count);

/* Projections of device vectors (no counterpart in the reference; its
 * Davidson forms them as separate dots, src/solvers/davidson.cpp:143-150,
 * 213-223): out[2 (o k + j)], out[2 (o k + j) + 1] = Re, Im <V_j, W_o> for
 * j < k, o < nw <= 4, where V_j = v_dev[j] and W_o = w_dev[o] are host arrays
 * of device pointers to n complex FP32 elements (16-byte aligned).
 * method 0: compensated CUDA-core kernel (FP64-accurate sums, k nw <= 4088);
 * method 1: tensor cores (tcgen05, each product as hi*hi + hi*lo + lo*hi of
 * TF32 splits, FP32 sums of about a thousand products added in FP64;
 * k <= 128; a pointer off the 16-byte grid is QKRYLOV_ERROR_INVALID_ARG);
 * method 2: CUDA cores, FP32 sums over runs of 32 elements folded into
 * float-float sums (error about 6 u of sum |v||w|, u = 2^-24; k nw <= 4088).
 * Every pointer must be 8-byte aligned (16-byte for method 1); others are
 * QKRYLOV_ERROR_INVALID_ARG.
 * Waits for `stream`.  Calls are serialised inside the library (one pointer
 * table and workspace per device, kept between calls). */
int qkrylov_vector_mdot_device_f32(const void* const* v_dev, int k, const void* const* w_dev, int nw, uint64_t n,
                                   int method, double* out, void* stream);
/* Combinations of device vectors, the update half of a block Gram-Schmidt
 * (no counterpart in the reference, whose Davidson subtracts one axpy per pair,
 * src/solvers/davidson.cpp:213-223): W_o = (accumulate ? W_o : 0) +
 * sum_j C_oj V_j for o < nw <= 8, j < k, k nw <= 1024, with
 * C_oj = coeffs[2 (o k + j)] + i coeffs[2 (o k + j) + 1] (rounded to FP32) and
 * FP32 sums in ascending j.  One pass over the V_j for all outputs; every
 * pointer 8-byte aligned (else QKRYLOV_ERROR_INVALID_ARG).  Returns
 * when the kernel has been queued on `stream` and the host arrays may be
 * reused. */
int qkrylov_vector_mcombine_device_f32(const void* const* v_dev, int k, const double* coeffs, void* const* w_dev,
                                       int nw, uint64_t n, int accumulate, void* stream);
/* Kernel the solvers' FP32 projections use (the mixed Davidson's projected
 * matrix and Gram-Schmidt passes): 0 the compensated CUDA-core kernel, 1 the
 * tensor-core kernel where it applies, 2 the run-summed CUDA-core kernel
 * (method 2 above; the default).  Process-wide. */
int qkrylov_set_projection_kernel(int method);

/* Test hooks (no counterpart in the reference).
 * qkrylov_debug_inject_alloc_failure: the after_n-th device allocation of the
 * library from now on (0: the next one) fails as cudaMalloc does on an
 * exhausted GPU; -1 switches the injection off.  Creators then return NULL and
 * other calls QKRYLOV_ERROR_CUDA, with qkrylov_last_error() set.
 * qkrylov_debug_live_allocations: device allocations the library holds now.
 * qkrylov_debug_device_wait_probe: one kernel waits on an mbarrier that nothing
 * completes, for limit_ns of GPU global time (clamped to 1 us .. 1 s), and
 * counts the give-up as qkrylov_device_wait_timeouts does; no copy is in
 * flight, the GPU stays usable. */
int qkrylov_debug_inject_alloc_failure(int64_t after_n);
int64_t qkrylov_debug_live_allocations(void);
int qkrylov_debug_device_wait_probe(int64_t limit_ns);

/* Select the GPU for Hamiltonians created afterwards on this thread (the
 * reference's Device(id), include/qkrylov/core/device.hpp:27-45), and wait for
 * all work on the current GPU. */
int qkrylov_set_device(int device_id);
int qkrylov_device_synchronize(void);
/* Visible CUDA devices (0 without a driver or device; the reference's
 * Device::gpu_count, include/qkrylov/core/device.hpp:71-84). */
int qkrylov_device_count(int* count);

int qkrylov_davidson_lowest_complex_f64(qkrylov_hamiltonian_h h, int n_eig, int max_subspace, double tol,
                                        double* eigenvalues_out, double* eigenvectors_complex_out,
                                        qkrylov_davidson_result_c_t* result_info);
/* Davidson with its diagnostics, in either form: mixed == 0 is the FP64
 * drop-in above; mixed != 0 keeps the Krylov vectors and the SpMV in FP32 with
 * FP64-accurate (compensated) projections and norms, and refines the returned
 * Ritz pairs in FP64 (Rayleigh quotient, residual).  max_iter: the
 * reference's 100 iterations, or fewer (1..100).  residuals (optional, n_eig):
 * ||H v - lambda v|| of the returned pairs; seconds (optional): wall time of
 * the solve. */
int qkrylov_davidson_lowest_ex(qkrylov_hamiltonian_h h, int n_eig, int max_subspace, double tol, int mixed,
                               int max_iter, double* eigenvalues, double* eigenvectors, double* residuals,
                               qkrylov_davidson_result_c_t* result_info, double* seconds);

int    qkrylov_continued_fraction_coeffs_complex_f64(qkrylov_hamiltonian_h h, const double* phi0_complex, int n_iter,
                                                     double* alphas_out, double* betas_out, double* norm_phi0_out,
                                                     int* num_coeffs_out, int* num_betas_out);
double qkrylov_evaluate_spectral_function_f64(const double* alphas, const double* betas, size_t n, double norm_phi0,
                                              double omega, double E0, double eta);
/* S(omega) on a whole grid: out[k] at omegas[k]. */
int    qkrylov_evaluate_spectral_grid_f64(const double* alphas, const double* betas, size_t n, double norm_phi0,
                                          const double* omegas, size_t n_omega, double E0, double eta, double* out);

typedef struct {
    double beta;
    double partition_function;
    double internal_energy;
    double specific_heat;
} qkrylov_ftlm_result_f64_t;

int qkrylov_ftlm_f64(qkrylov_hamiltonian_h h, double beta, int n_random, int n_steps, qkrylov_ftlm_result_f64_t* result);
/* One FTLM run (the reference's random vectors, ftlm.cpp:133-148) evaluated at
 * n_beta inverse temperatures.  If log_shift is non-NULL the weights use
 * exp(-beta (E - E_min)) and log_shift[k] = -beta_k E_min, so that
 * Z_k = partition_function_k * exp(log_shift[k]) stays finite where the
 * reference's exp(-beta E) overflows. */
int qkrylov_ftlm_multi_beta_f64(qkrylov_hamiltonian_h h, const double* betas, int n_beta, int n_random, int n_steps,
                                double* Z_out, double* E_out, double* Cv_out, double* log_shift);

/* Compile statistics of a Hamiltonian: terms per kernel class and diagonal
 * storage (0: 1-byte code, 1: 2-byte code, 2: full). */
int qkrylov_hamiltonian_info(qkrylov_hamiltonian_h h, int* n_outer, int* n_inner, int* n_mixed, int* n_diag,
                             int* diag_mode);

/* SpMV kernel choice: generic = 0 lets the library use its table-driven fast
 * kernel when the Hamiltonian qualifies (32-bit states, coded diagonal), in
 * the variant its autotuner measured fastest at creation; generic = 1 forces
 * the generic kernel; 2 the fast kernel with one row per thread; 3 the fast
 * kernel with shared-memory staging of each outer block's slice of x (when a
 * block fits); 4 the fast kernel with four rows per thread; 5 four rows per
 * thread with the block staged (when it fits); 6 four rows per thread with a
 * larger register budget; 7, 8, 9 the tiled kernel over 1, 2, 4 outer blocks
 * per CTA (the blocks' slices of x in shared memory; when they fit); 10 the
 * class-persistent kernel (one CTA per SM, inner table and slices of x in
 * shared memory; when they fit).
 * *fast_in_use (optional) reports whether the fast kernel applies. */
int qkrylov_hamiltonian_select_kernel(qkrylov_hamiltonian_h h, int generic, int* fast_in_use);

/* The fast-kernel variant mode 0 uses for FP32 (fp32 != 0) or FP64 vectors
 * (*variant: 0 one row per thread, 1 staged, 2 four rows per thread, 3 four
 * rows per thread staged, 4 four rows per thread wide; -1 when the generic kernel
 * applies) and the autotuner's mean launch times per variant
 * (ms_per_variant[5], 0 = not measured; sectors below 2^20 rows are not
 * timed).  *variant is 5 when mode 0 uses a variant added later (see
 * qkrylov_hamiltonian_tuning_ex). */
int qkrylov_hamiltonian_tuning(qkrylov_hamiltonian_h h, int fp32, int* variant, double* ms_per_variant);

/* The same with every variant: *variant 0..4 as above, 5, 6, 7 the tiled
 * kernel over 1, 2, 4 outer blocks per CTA, 8 the class-persistent kernel; ms_per_variant receives n_ms
 * entries (variants beyond those the library has read 0). */
int qkrylov_hamiltonian_tuning_ex(qkrylov_hamiltonian_h h, int fp32, int* variant, double* ms_per_variant, int n_ms);

/* States first .. first + count - 1 of a basis in the reference's order and
 * bit encoding (qkrylov_basis_state for a range). */
int qkrylov_basis_states(qkrylov_basis_h basis, uint64_t first, uint64_t count, uint64_t* out);

/* Device memory the Hamiltonian keeps between solver calls (the FP32 Krylov
 * space of the mixed Lanczos: maxiter + 7 vectors): *bytes receives its size;
 * release != 0 frees it now (it is also freed with the Hamiltonian). */
int qkrylov_hamiltonian_workspace(qkrylov_hamiltonian_h h, int release, uint64_t* bytes);

/* Time `reps` back-to-back applies of the FP32 (fp32 != 0) or FP64 kernel on
 * internal device vectors, with CUDA events on the Hamiltonian's stream;
 * *ms_per_apply receives the mean launch duration. */
int qkrylov_hamiltonian_benchmark_apply(qkrylov_hamiltonian_h h, int fp32, int reps, double* ms_per_apply);

/* Every generated matrix entry, rows and columns in the reference's order and
 * entries of a row in OpSum term order -- the content of the reference's CSR
 * (matrix_free_hamiltonian.cpp:45-92).  Call once with row_offsets = cols =
 * vals = NULL to get *nnz_out, then again with arrays of dim+1, nnz and 2*nnz. */
int qkrylov_hamiltonian_entries(qkrylov_hamiltonian_h h, uint64_t* nnz_out, uint64_t* row_offsets, uint64_t* cols,
                                double* vals);

/* ---- batched Lanczos over block vectors (GB300 additions) -------------------
 * Several Hamiltonians (e.g. every Sz sector of one chain) with n_vec vectors
 * each are advanced together: every Lanczos step is one block-SpMV launch for
 * all of them (vectors interleaved by row), with all scalars on the device and
 * the steps replayed as a CUDA graph.  The recurrence per vector is the
 * reference's compute_tridiag / continued_fraction_coeffs loop
 * (src/solvers/ftlm.cpp:24-53, src/solvers/dynamics.cpp:13-59), including its
 * stop at beta < 1e-15.  mixed != 0: FP32 vectors and SpMV, compensated
 * reductions combined in FP64; mixed == 0: FP64 throughout.  Needs every
 * Hamiltonian on the fast SpMV kernel (32-bit states) and on one device. */
#define QKRYLOV_START_FTLM_STREAM 0     /* mt19937(42) complex normal per Hamiltonian (ftlm.cpp:133-143) */
#define QKRYLOV_START_PHILOX 1          /* seeded Philox Gaussian vectors generated on the device */
#define QKRYLOV_START_GIVEN 2           /* caller's vectors, reference order */
#define QKRYLOV_START_FTLM_STREAM_F32 3 /* the FTLM stream through normal_distribution<float> */

typedef struct {
    double seconds;         /* device time of the Lanczos loop (CUDA events; start vectors excluded) */
    double spmv_ms;         /* mean CUDA-event time of one block SpMV launch (first steps) */
    int vectors_per_lane;   /* block-SpMV tile shape picked by the autotuner (1, 2 or 4) */
    int padded_vectors;     /* vectors per row in the block (n_vec rounded up to a power of two) */
    uint64_t rows;          /* sum of the Hamiltonians' dimensions */
    double tune_ms[3];      /* autotuner timings for 1, 2, 4 vectors per lane (0: not measured) */
} qkrylov_block_stats_t;

/* Tridiagonals of n_ham * n_vec vectors (vector i = h * n_vec + v), n_steps
 * steps each.  start_vectors (QKRYLOV_START_GIVEN): for each Hamiltonian in
 * order, n_vec vectors of its dimension, complex interleaved [re, im].
 * alphas/betas: [i * n_steps + k]; n_alpha/n_beta: counts recorded per vector;
 * norm2: squared norm of each start vector.  vectors_per_lane: block-SpMV
 * tile (1, 2 or 4 vectors per lane; 0 = autotuned).  stats is optional. */
int qkrylov_block_lanczos_tridiag(const qkrylov_hamiltonian_h* hams, int n_ham, int n_vec, int n_steps, int mixed,
                                  int vectors_per_lane, int start_kind, uint64_t seed, const double* start_vectors,
                                  double* alphas,
                                  double* betas, int* n_alpha, int* n_beta, double* norm2,
                                  qkrylov_block_stats_t* stats);

/* FTLM (ftlm.cpp:123-170) summed over Hamiltonians: Z = sum_h Z_h,
 * E = sum_h Z_h E_h / Z, Cv = beta^2 (<E^2> - <E>^2), n_random vectors per
 * Hamiltonian (<= 32) in one batched run, evaluated at n_beta inverse
 * temperatures.  log_shift (optional, n_beta): shifted evaluation, the true
 * partition function is Z * exp(log_shift). */
int qkrylov_ftlm_sectors_f64(const qkrylov_hamiltonian_h* hams, int n_ham, const double* betas, int n_beta,
                             int n_random, int n_steps, int mixed, int start_kind, uint64_t seed, double* Z, double* E,
                             double* Cv, double* log_shift, qkrylov_block_stats_t* stats);

/* Continued-fraction coefficients (dynamics.cpp:13-59) of n_rhs right-hand
 * sides (<= 32; phi0: n_rhs vectors of the Hamiltonian's dimension, reference
 * order, complex interleaved) in one batched run.  alphas/betas
 * [r * n_iter + k], n_alpha/n_beta counts, norms: ||phi0_r|| (0 for a zero
 * vector, which gets no coefficients). */
int qkrylov_cf_block_f64(qkrylov_hamiltonian_h h, const double* phi0, int n_rhs, int n_iter, int mixed,
                         double* alphas, double* betas, int* n_alpha, int* n_beta, double* norms,
                         qkrylov_block_stats_t* stats);

#ifdef __cplusplus
}
#endif

#endif /* QKRYLOV_GB300_C_API_H */
