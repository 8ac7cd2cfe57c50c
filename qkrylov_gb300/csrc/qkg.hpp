// Internal declarations shared by the host C++ and the CUDA translation units
// of libqkrylov_gb300.  Nothing here is part of the public C ABI
// (include/qkrylov_c_api.h).
#pragma once

#include <cuda_runtime.h>

#include <complex>
#include <cstdint>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

namespace qkg {

// ---------------------------------------------------------------- errors
// Status codes of the C ABI: 0, -1, -2 keep the reference's meaning
// (include/qkrylov/c_api.h:14-16); -3 and -4 are additions of this library.
enum Status : int { OK = 0, INVALID_ARG = -1, EXCEPTION = -2, CUDA_ERR = -3, DEVICE_TIMEOUT = -4 };

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

void set_last_error(const std::string& msg);
const char* last_error();

#define QKG_CUDA(call)                                                                                  \
    do {                                                                                               \
        cudaError_t e_ = (call);                                                                       \
        if (e_ != cudaSuccess)                                                                         \
            throw ::qkg::Error(::qkg::CUDA_ERR, std::string(#call) + ": " + cudaGetErrorString(e_));   \
    } while (0)
// Every kernel launch site ends with QKG_LAUNCHED(): it counts the launch
// (qkrylov_kernel_launches()) and surfaces launch errors.
void count_launch();
uint64_t launch_count();
// Graph capture records launches without running them: the capturing code
// takes them back (negative d) and adds the graph's kernels per replay.
void add_launches(int64_t d);
#define QKG_LAUNCHED()                                                                                      \
    do {                                                                                                   \
        ::qkg::count_launch();                                                                             \
        const cudaError_t le_ = cudaGetLastError();                                                        \
        if (le_ != cudaSuccess)                                                                            \
            throw ::qkg::Error(::qkg::CUDA_ERR, std::string("kernel launch at ") + __FILE__ + ":" +         \
                                                    std::to_string(__LINE__) + ": " + cudaGetErrorString(le_)); \
    } while (0)
// Device memory of the library goes through device_alloc/device_free: they
// count the live allocations (qkrylov_debug_live_allocations) and let a test
// make the n-th allocation fail as cudaMalloc would on an exhausted GPU
// (qkrylov_debug_inject_alloc_failure).
void device_alloc(void** p, size_t bytes);
void device_free(void* p);
int64_t live_device_allocs();
void inject_alloc_failure(int64_t after_n);
#define QKG_REQUIRE(cond, msg)                                                \
    do {                                                                      \
        if (!(cond)) throw ::qkg::Error(::qkg::INVALID_ARG, std::string(msg)); \
    } while (0)

// ---------------------------------------------------------------- model
enum Model : int { SPIN = 0, FERMION = 1, HUBBARD = 2, TJ = 3 };

// Sector flags; same fields and meaning as the reference's Sector
// (include/qkrylov/symmetry/sector.hpp:10-41).
struct Sector {
    bool use_sz = false; int sz2 = 0;
    bool use_nup = false, use_ndn = false; int nup = 0, ndn = 0;
    bool use_n = false; int n = 0;
    bool use_nb = false; int nb = 0;
};

// Two ways of ranking an internal state on the device.
enum RankKind : int { RANK_TABLE = 0, RANK_SEARCH = 1 };

// Device copy of a basis' rank/unrank tables (one per GPU that used the basis).
struct DevBasis {
    int nbits = 0, n_in = 0, n_out = 0, rank_kind = RANK_TABLE;
    int N = 0, split = 0, inner_all = 0, idx32 = 0;
    uint64_t in_mask = 0, dim = 0;
    // popcount constraint groups (internal encoding) and the t-J rule
    int ngroups = 0, no_double = 0;
    uint64_t gmask[2] = {0, 0};
    int gpop[2] = {0, 0};
    const void* outer_off = nullptr;      // uint32 (idx32) or uint64, 2^n_out + 1 entries
    const uint32_t* inner_rank = nullptr;   // 2^n_in entries (null if inner_all)
    const uint32_t* inner_state = nullptr;  // class-ordered inner configurations
    const uint64_t* states_int = nullptr;   // sorted internal states (RANK_SEARCH)
    const void* ref_of_int = nullptr;       // reference index of each internal index (permuted bases)
};

// A span of consecutive rows inside one outer block.
struct WorkItem {
    uint64_t row0;
    uint32_t count;
    uint32_t a;           // outer configuration (RANK_TABLE)
    uint32_t inner_base;  // index into inner_state of the first row's inner configuration
    uint32_t pad;
};

class Basis {
public:
    Basis(Model m, int N, const Sector& sec);
    ~Basis();

    Model model;
    int N;
    Sector sec;
    int nbits;        // bits of one state in either encoding (N, or 2N for Hubbard/t-J)
    bool split;       // internal encoding puts up bits at 0..N-1 and down bits at N..2N-1
    bool permuted;    // internal order differs from the reference order
    uint64_t dim = 0;

    int ngroups = 0;
    uint64_t gmask[2] = {0, 0};
    int gpop[2] = {0, 0};
    bool no_double = false;

    int rank_kind = RANK_TABLE;
    int n_in = 0, n_out = 0;
    bool inner_all = false;
    int inner_fixed_class = -1;  // fixed inner popcount class, or -1
    uint64_t in_mask_ = 0;
    int total_pop = -1;          // spin/fermion fixed total popcount (inner class = total - pop(a))
    std::vector<uint64_t> outer_off;
    std::vector<uint32_t> inner_rank, inner_state, class_base;
    // spin/fermion bases whose inner order is not colex: the colex (reference)
    // rank of each inner configuration and the colex-ordered configurations
    std::vector<uint32_t> ref_inner_rank, ref_inner_state;
    std::vector<uint64_t> states_int;  // RANK_SEARCH
    std::vector<uint64_t> states_ref;  // t-J only: sorted reference-encoded states

    // encodings
    uint64_t to_internal(uint64_t s_ref) const;
    uint64_t to_reference(uint64_t s_int) const;
    bool contains_int(uint64_t s) const;
    uint64_t rank_int(uint64_t s) const;    // requires contains_int(s)
    uint64_t unrank_int(uint64_t i) const;  // i < dim
    int inner_class_of(uint32_t a) const;   // -1 if block a is empty
    uint64_t block_size(uint32_t a) const;

    // reference-facing queries (reference encoding and order)
    bool contains_ref(uint64_t s_ref) const;
    int64_t index_ref(uint64_t s_ref) const;
    uint64_t state_ref(uint64_t i_ref) const;
    uint64_t ref_index_of_int(uint64_t i_int) const;

    std::vector<WorkItem> work_items(uint32_t chunk) const;

    // device copy, built on first use on a device
    const DevBasis& device(int dev);

private:
    bool inner_reordered_ = false;  // inner classes are not in colex order
    struct DevCopy;
    std::mutex mu_;
    std::vector<std::unique_ptr<DevCopy>> dev_;
};

uint64_t binom(int n, int k);

// Reference index of every internal index, computed on the device from the
// work items (out: uint32 when idx32, else uint64).  Split (Hubbard) bases use
// the interleaved count; spin/fermion bases pass the colex rank of each inner
// configuration (ref_inner_rank, 2^n_in entries).
void ref_permutation_device(const DevBasis& d, const Sector& sec, const std::vector<WorkItem>& items,
                            const std::vector<uint32_t>* ref_inner_rank, void* out);

// ---------------------------------------------------------------- operators
struct Factor { std::string op; int site; };
struct Term { std::complex<double> coeff; std::vector<Factor> factors; };

// A factor whose amplitude depends on bits that no condition fixes:
// amplitude = ((s ^ pf) & sm) == sm ? a1 : a0, on the original row state s.
struct DVar { uint64_t sm, pf; double a0r, a0i, a1r, a1i; };

// One OpSum term compiled for the internal encoding.  For a row state s the
// term is valid iff (s & C) == V; it maps s to s ^ X; the stored amplitude is
// the complex conjugate of the reference's amp (rows store conj(amp),
// src/hamiltonian/matrix_free_hamiltonian.cpp:75-84), times
// (-1)^popcount(s & J) and the variable factors.
template <class S>
struct DTerm {
    S C, V, X, J;
    double ar, ai;
    uint32_t flags;  // bit 0: target needs a basis-membership check; bits 8..15: number of variable factors
    uint32_t var0;   // first variable factor in the DVar array
};

struct HostTerm {  // state-width independent form, built on the host
    uint64_t C = 0, V = 0, X = 0, J = 0;
    std::complex<double> amp;  // already conjugated
    bool check = false;
    std::vector<DVar> vars;
    int src = 0;               // index of the OpSum term it came from
};

enum SiteKind : int { SITE_SPIN = 0, SITE_FERMION = 1, SITE_HUBBARD = 2, SITE_TJ = 3 };

// Compile an OpSum for a basis and a site kind.  Dead terms (never valid on
// the basis) are dropped; unknown operators and sites outside [0, 64) for the
// site's bit layout throw Error(INVALID_ARG).
std::vector<HostTerm> compile_terms(const Basis& b, SiteKind site, const std::vector<Term>& terms);

}  // namespace qkg
