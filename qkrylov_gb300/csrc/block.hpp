// Batched three-term Lanczos over block vectors: R vectors per Hamiltonian
// (FTLM random vectors, continued-fraction right-hand sides) for one or more
// Hamiltonians (e.g. every Sz sector of a chain) advanced together, one block
// SpMV launch per step for all of them.
#pragma once

#include "ham.hpp"

#include <complex>
#include <vector>

namespace qkg {

enum class BlockStart {
    FtlmStream,  // the reference FTLM stream per Hamiltonian: mt19937(42), complex normal (ftlm.cpp:133-143)
    Philox,      // seeded Philox Gaussian vectors generated on the device
    Given,       // caller's vectors, reference order
};

struct BlockOpts {
    int R = 1;            // vectors per Hamiltonian (padded to a power of two <= 32 inside)
    int steps = 100;      // Lanczos steps per vector
    bool mixed = true;    // FP32 vectors and SpMV with compensated reductions; else FP64
    BlockStart start = BlockStart::FtlmStream;
    uint64_t seed = 0;
    bool f32_stream = false;           // FtlmStream through the float distribution
    std::vector<const std::complex<double>*> given;  // Given: [h * R + r], reference order
    int vpl = 0;          // vectors per lane of the block SpMV (0: autotuned)
};

// Per vector v = h * R + r: its tridiagonal (the alphas and betas the
// reference's compute_tridiag / continued_fraction_coeffs record: the loop
// stops when beta < 1e-15, ftlm.cpp:36-52, dynamics.cpp:38-56) and the squared
// norm of its start vector.
struct BlockTridiag {
    int n_ham = 0, R = 0, steps = 0;
    std::vector<std::vector<double>> alpha, beta;
    std::vector<double> norm2;
    double seconds = 0.0;        // device time of the Lanczos loop (CUDA events; start vectors excluded)
    double spmv_ms = 0.0;        // mean CUDA-event time of the timed block-SpMV launches
    int vpl = 0;                 // vectors per lane used
    int rp = 0;                  // padded vectors per row
    uint64_t rows = 0;           // total rows of the block vector (sum of dimensions)
    std::vector<double> tune_ms; // autotuner record per vpl 1, 2, 4 (0 = not measured)
};

BlockTridiag block_lanczos(const std::vector<Hamiltonian*>& hs, const BlockOpts& o);

// FTLM observables over several Hamiltonians (sum of the per-Hamiltonian
// estimates of ftlm.cpp:151-167, R vectors each): Z = sum_h Z_h,
// E = sum_h Z_h E_h / Z, Cv = beta^2 (<E^2> - <E>^2).  With `shifted` the
// weights use exp(-beta (e - e_min)) over all Hamiltonians and log_zmax[b] =
// -beta e_min.
void ftlm_observables_block(const BlockTridiag& t, const double* betas, int nb, double* Z, double* E, double* Cv,
                            bool shifted, double* log_zmax);

}  // namespace qkg
