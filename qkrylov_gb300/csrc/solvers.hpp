// Solver drivers: host loops over device-resident Krylov state.
#pragma once

#include "ham.hpp"

#include <complex>
#include <random>
#include <vector>

namespace qkg {

using cd = std::complex<double>;

// ---- small dense eigenproblems (host, FP64) ---------------------------------
// Lowest eigenvalue of the symmetric tridiagonal (a[0..n-1], b[0..n-2]) by
// Sturm-sequence bisection.
double tridiag_lowest(const double* a, const double* b, int n);
// All eigenvalues and the rows of the eigenvector matrix listed in `rows`
// (implicit-shift QL with Wilkinson shifts).  z[r*n + j] = component `rows[r]`
// of eigenvector j.
void tridiag_eig(const double* a, const double* b, int n, std::vector<double>& evals, const std::vector<int>& rows,
                 std::vector<double>& z);
// Lowest eigenvalue and its eigenvector (full vector, length n): Sturm
// bisection and inverse iteration, O(n); _ql: the same by QL, O(n^3).
double tridiag_ground(const double* a, const double* b, int n, std::vector<double>& vec);
double tridiag_ground_ql(const double* a, const double* b, int n, std::vector<double>& vec);
// Eigenvector for the eigenvalue lam by inverse iteration (false: breakdown).
bool tridiag_vector(const double* a, const double* b, int n, double lam, std::vector<double>& vec);
// Selective orthogonalisation (Parlett & Scott, Math. Comp. 33 (1979)): the
// Ritz values among the max_locked (<= kMaxRitzLocked) lowest of T_k whose residual estimate
// |beta_k s_{k,i}| <= tol ||T|| and that are not yet in `locked` (within
// tol ||T||), ascending; later Lanczos vectors are kept orthogonal to their
// Ritz vectors.
constexpr int kMaxRitzLocked = 4;
std::vector<double> ritz_to_lock(const double* a, const double* b, int k, double beta, double tol,
                                 const std::vector<double>& locked, int max_locked = kMaxRitzLocked);
// Hermitian m x m eigenproblem (cyclic complex Jacobi), ascending eigenvalues;
// vecs[k][i] = component i of eigenvector k.
void hermitian_eig(const std::vector<cd>& H, int m, std::vector<double>& evals, std::vector<std::vector<cd>>& vecs);

// ---- reference random streams (host) -----------------------------------------
// Filled as the reference fills KComplex(dist(rng), dist(rng)) when compiled
// with g++, which evaluates the imaginary (second) argument first
// (src/solvers/lanczos.cpp:115-120, ftlm.cpp:133-143, davidson.cpp:106-128).
// `f32` draws through the float distributions, as the reference's FP32 engine
// (the one behind its C API, where Real = float) does.
void ref_uniform_complex(uint32_t seed, uint64_t n, cd* out, bool f32 = false);
template <class Dist>
void fill_stream(std::mt19937& rng, Dist& dist, uint64_t n, cd* out) {
    for (uint64_t i = 0; i < n; ++i) {
        const double im = dist(rng);  // g++ evaluates the imaginary argument first
        const double re = dist(rng);
        out[i] = cd(re, im);
    }
}
// The FTLM random stream: one mt19937(42) normal stream across all vectors of
// one run (src/solvers/ftlm.cpp:133-143).
struct NormalStream {
    std::mt19937 rng{42};
    std::normal_distribution<double> d64{0.0, 1.0};
    std::normal_distribution<float> d32{0.0f, 1.0f};
    bool f32;
    explicit NormalStream(bool f) : f32(f) {}
    void fill(uint64_t n, cd* out) {
        if (f32) fill_stream(rng, d32, n, out);
        else fill_stream(rng, d64, n, out);
    }
};
// Device Philox4x32-10 (Salmon et al., SC'11) Gaussian complex vectors.
void philox_normal_f64(uint64_t seed, uint64_t stream, double2* out, uint64_t n, cudaStream_t s);
void philox_normal_f32(uint64_t seed, uint64_t stream, float2* out, uint64_t n, cudaStream_t s);

// ---- Lanczos -------------------------------------------------------------------
struct LanczosOpts {
    int maxiter = 200;
    double tol = 1e-12;
    bool want_vec = false;
    const cd* v0_ref = nullptr;  // start vector in reference order (else the reference's RNG stream)
    bool fixed_steps = false;    // run exactly maxiter steps (no early exit on |dE| < tol)
    bool device_start = false;   // seeded Philox Gaussian start (performance runs)
    uint64_t seed = 0;
    bool f32_stream = false;     // draw the start vector as the reference's FP32 engine does
    cd* evec_out = nullptr;      // with want_vec: the Ritz vector goes here (reference order) instead of LanczosOut::evec
    bool selective = false;      // FP64 form: selective instead of full reorthogonalisation (the mixed form's scheme)
    int ritz_guard = 1;          // selective reorthogonalisation guards the converged Ritz vectors among the
                                 // ritz_guard lowest (the wanted end: 1 for a ground state, <= kMaxRitzLocked)
};
struct LanczosOut {
    double energy = 0.0;       // reported energy (refined for the mixed form)
    double energy_tridiag = 0.0;
    double residual = 0.0;     // ||H psi - E psi|| (FP64) when computed, else -1
    int iters = 0;
    bool converged = false;
    std::vector<double> alphas, betas;
    std::vector<cd> evec;      // reference order
    double t_loop = 0.0;       // seconds in the Lanczos loop (device-synchronised)
    double t_refine = 0.0;
    int n_selective = 0;       // steps that were re-orthogonalised against converged Ritz vectors
    int n_ritz_locked = 0;     // converged Ritz vectors held at the end (selective reorthogonalisation)
    double t_spmv = 0.0;       // summed CUDA-event time of the loop's SpMV launches (seconds)
    int n_spmv = 0;
};

// CUDA-event timer for launches on one stream; elapsed time is collected
// after the stream has been synchronised by the caller.
class LaunchTimer {
public:
    explicit LaunchTimer(cudaStream_t s);
    ~LaunchTimer();
    void start();
    void stop();      // records the end event
    double collect(); // seconds between the last start/stop pair (stream must be past it)
private:
    cudaStream_t s_;
    cudaEvent_t a_ = nullptr, b_ = nullptr;
};
// Plain FP64 path with the reference's semantics (full reorthogonalisation,
// convergence when |E_k - E_{k-1}| < tol; src/solvers/lanczos.cpp:101-202).
LanczosOut lanczos_f64(Hamiltonian& H, const LanczosOpts& o);
// Mixed form: FP32 vectors and SpMV, compensated reductions combined in FP64,
// selective reorthogonalisation against the converged Ritz vector, FP64
// Rayleigh-quotient + residual refinement at the end.
LanczosOut lanczos_mixed(Hamiltonian& H, const LanczosOpts& o);
// The same mixed form with a device-resident recurrence (one CUDA graph per
// step); needs the fast SpMV kernel and room for maxiter + 1 FP32 vectors.
bool lanczos_device_supported(const Hamiltonian& H);
// device memory a device-resident mixed run of maxiter steps holds
size_t lanczos_device_bytes(const Hamiltonian& H, int maxiter);
LanczosOut lanczos_mixed_device(Hamiltonian& H, const LanczosOpts& o);

// ---- continued fraction (src/solvers/dynamics.cpp:13-89) --------------------------
struct CFOut { std::vector<double> alphas, betas; double norm = 0.0; };
CFOut cf_f64(Hamiltonian& H, const cd* phi0_ref, int n_iter);
double spectral(const double* alphas, const double* betas, size_t n, double norm, double omega, double E0, double eta);

// ---- FTLM (src/solvers/ftlm.cpp:123-170) ---------------------------------------
struct FTLMTri {  // per random vector
    std::vector<double> evals, w0;  // eigenvalues and squared first components
    double norm2 = 0.0;             // ||r||^2 of the un-normalised random vector
};
std::vector<FTLMTri> ftlm_tridiags_f64(Hamiltonian& H, int n_random, int n_steps, bool f32_stream = false);
void ftlm_observables(const std::vector<FTLMTri>& tri, const double* betas, int nb, double* Z, double* E, double* Cv,
                      bool shifted, double* log_zmax);

// ---- Davidson (src/solvers/davidson.cpp:86-227) -------------------------------
struct DavidsonOut {
    std::vector<double> evals;
    std::vector<std::vector<cd>> evecs;
    int iters = 0;
    bool converged = false;
    std::vector<double> residuals;  // ||H v - lambda v|| of the returned pairs (FP64 for the mixed form)
    double seconds = 0.0;
};
// max_iter: the reference's fixed 100 iterations (davidson.cpp:141,180) unless
// a caller asks for fewer (timing runs).
DavidsonOut davidson_f64(Hamiltonian& H, int n_eig, int max_sub, double tol, bool want_vecs, bool f32_stream = false,
                         int max_iter = 100);
// Mixed form: FP32 Krylov vectors and SpMV, FP64-accurate (compensated) projections
// and norms, FP64 Rayleigh-quotient and residual refinement of the Ritz pairs.
DavidsonOut davidson_mixed(Hamiltonian& H, int n_eig, int max_sub, double tol, bool want_vecs, int max_iter = 100);

}  // namespace qkg
